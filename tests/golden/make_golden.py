"""Generate the golden fixtures that pin the oracle to the AdaM-DG reference.

Runs oracle/_ref/ref_harness (the reference library compiled from its own
sources, see oracle/Makefile) and stores its outputs, keyed by element
multi-index, as small .npz files in this directory.  Run in a tree that has
the reference checkout:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def parse_harness(text: str) -> dict:
    """Parse BEGIN/END blocks, META and scalar lines of ref_harness output."""
    out: dict = {"meta": {}}
    lines = text.splitlines()
    i = 0
    while i < len(lines):
        ln = lines[i].strip()
        if ln.startswith("BEGIN"):
            _, name, rows, cols = ln.split()
            rows, cols = int(rows), int(cols)
            data = np.array([[float(v) for v in lines[i + 1 + r].split()] for r in range(rows)]).reshape(rows, cols)
            out[name] = data
            i += rows + 2
            continue
        if ln.startswith("META"):
            for kv in ln.split()[1:]:
                k, v = kv.split("=")
                out["meta"][k] = int(v)
        elif ln.startswith("NORMERR"):
            f = ln.split()
            out.setdefault("normerr", {})[int(f[1])] = [float(v) for v in f[2:5]]
        elif ln.startswith("L2ERR"):
            out["l2err"] = float(ln.split()[1])
        elif ln.startswith("TIME"):
            for kv in ln.split()[1:]:
                k, v = kv.split("=")
                out["meta"][k] = float(v)
        i += 1
    return out


def split_elements(block: np.ndarray, dim: int):
    level = block[:, :dim].astype(np.int32)
    suppt = block[:, dim:2 * dim].astype(np.int32)
    coef = block[:, 2 * dim:]
    return level, suppt, coef


def run(args):
    res = subprocess.run([HARNESS] + [str(a) for a in args], check=True, capture_output=True, text=True)
    return parse_harness(res.stdout)


# (name, dim, N, k, ic, engine, steps, dt, c)
LINEAR_CASES = [
    ("lin2d_n4_sinsum", 2, 4, 2, "sin_sum", "assembled", 5, 0.005, [1.0, 1.0]),
    ("lin2d_n5_mixedc", 2, 5, 2, "sin_sum", "assembled", 3, 0.002, [1.0, -0.5]),
    ("lin2d_n7_config1", 2, 7, 2, "sin_sum", "assembled", 4, 1.0 / 2561.0, [1.0, 1.0]),
    ("lin3d_n4_sinprod", 3, 4, 2, "sin_prod", "assembled", 3, 0.004, [1.0, 1.0, 1.0]),
    ("lin4d_n3_matfree", 4, 3, 2, "sin_prod", "matfree", 2, 0.005, [1.0, 1.0, 1.0, 1.0]),
    ("lin2d_n4_k1", 2, 4, 1, "sin_sum", "assembled", 3, 0.005, [1.0, 1.0]),
    ("lin2d_n3_k3", 2, 3, 3, "sin_sum", "assembled", 3, 0.005, [0.7, -1.3]),
]


# (name, dim, N, alpha, steps, dt): Lagrange-interpolated Burgers, LxF, SSP-RK3
BURGERS_CASES = [
    ("burgers2d_n4", 2, 4, 1.1, 2, 0.002),
    ("burgers3d_n4", 3, 4, 0.825, 2, 0.001),
    ("burgers3d_n5", 3, 5, 0.825, 1, 0.0005),
]


# (name, dim, n_init, nmax, eps, eta, alpha, cfl, umax, steps): adaptive Burgers time loop
BURGERS_ADAPT_CASES = [
    ("burgers_adapt2d", 2, 3, 7, 1e-4, 1e-5, 0.825, 0.1, 0.75, 4),
    ("burgers_adapt3d", 3, 3, 6, 3e-5, 3e-6, 0.825, 0.1, 0.75, 2),
]


# (name, dim, n_init, nmax, eps, eta, alpha, cfl, umax, steps, snapshot steps): the adaptive Burgers
# time loop at full length -- the 3D configuration of the benchmark (start level 3, max level 8,
# refine 1e-5, coarsen 1e-6, LxF alpha 0.825, CFL 0.1, 36 steps of 1/720 to T = 0.05).  The element
# set and three checksums of the coefficients are kept after every step, the coefficients themselves
# after the snapshot steps (0 = after the adaptive initialisation).
BURGERS_ADAPT_LONG_CASES = [
    ("burgers_adapt3d_config3", 3, 3, 8, 1e-5, 1e-6, 0.825, 0.1, 0.75, 36, [0, 1, 2, 9, 18, 27, 36]),
]


def checksum_weights(level: np.ndarray, suppt: np.ndarray, nb: int) -> np.ndarray:
    """Weights of the position-dependent checksum sum_e,i w(e, i) u[e, i]: a function of the
    element's level and support index and of the coefficient index only, so it does not depend on
    the order in which a run lists its elements."""
    dim = level.shape[1]
    h = np.zeros(len(level), np.int64)
    for d in range(dim):
        h = h * 131 + level[:, d].astype(np.int64) * 17 + suppt[:, d].astype(np.int64) * 5 + d
    w = (h[:, None] * 7 + np.arange(nb)[None, :] * 31) % 97
    return 0.5 + w / 97.0


def checksums(level: np.ndarray, suppt: np.ndarray, u: np.ndarray) -> np.ndarray:
    """[sum of squares, max |u|, weighted sum, sum of |weight * u|] of a coefficient field."""
    w = checksum_weights(level, suppt, u.shape[1])
    return np.array([float((u * u).sum()), float(np.abs(u).max()), float((w * u).sum()), float(np.abs(w * u).sum())])


# (name, dim, N, k, ic, engine, steps, dt, c): the linear advection case at its full length -- 2D,
# full sparse grid N = 7, CFL 0.1 (dt = 1/2561), 2561 SSP-RK3 steps to T = 1; initial and final
# coefficients and the final L1/L2/Linf errors against the exact translated solution (1 and 2
# Gauss points)
LINEAR_LONG_CASES = [
    ("lin2d_n7_config1_T1", 2, 7, 2, "sin_sum", "assembled", 2561, 1.0 / 2561.0, [1.0, 1.0]),
]


def linear_long(manifest):
    for name, dim, N, k, ic, engine, steps, dt, c in LINEAR_LONG_CASES:
        r = run(["linear", dim, N, k, 1, ic, engine, steps, repr(dt)] + [repr(x) for x in c])
        lv, sp, u0 = split_elements(r["u0"], dim)
        lv3, sp3, uT = split_elements(r["uT"], dim)
        assert (lv == lv3).all() and (sp == sp3).all()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), level=lv, suppt=sp, u0=u0, uT=uT,
                            **{f"normerr_g{gp}": np.array(err) for gp, err in r["normerr"].items()})
        manifest[name] = dict(kind="linear_long", dim=dim, N=N, k=k, ic=ic, engine=engine, steps=steps, dt=dt, c=c,
                              elements=int(r["meta"]["elements"]), normerr_g2=r["normerr"][2])
        print(name, r["meta"], r["normerr"])


# (name, dim, N_init, NMAX, eps, eta, sigma, cfl, steps, snapshot steps): the adaptive wave loop
# over 24 steps at max level 7 (refine 1e-5, coarsen 1e-6, start level 3): the element set and the
# checksums of u and u_t after every step, u and u_t themselves at the snapshot steps
WAVE_ADAPT_LONG_CASES = [
    ("wave_adapt2d_n7_long", 2, 3, 7, 1e-5, 1e-6, 10.0, 0.1, 24, [0, 1, 12, 24]),
]


def wave_adapt_long(manifest):
    for name, dim, n0, nmax, eps, eta, sigma, cfl, steps, snaps in WAVE_ADAPT_LONG_CASES:
        res = subprocess.run([HARNESS, "wave_adapt"] + [str(a) for a in (dim, n0, nmax, repr(eps), repr(eta),
                                                                          repr(sigma), repr(cfl), steps)],
                             check=True, capture_output=True, text=True)
        r = parse_harness(res.stdout)
        arrs, sums, elements = {}, [], []
        for i, tag in enumerate(["init"] + [f"step{s}" for s in range(steps)]):
            lv, sp, u = split_elements(r["u_" + tag], dim)
            lv2, sp2, ut = split_elements(r["ut_" + tag], dim)
            assert (lv == lv2).all() and (sp == sp2).all()
            arrs[f"level_{i}"], arrs[f"suppt_{i}"] = lv.astype(np.int16), sp.astype(np.int16)
            sums.append(np.concatenate([checksums(lv, sp, u), checksums(lv, sp, ut)]))
            elements.append(int(len(lv)))
            if i in snaps:
                arrs[f"u_{i}"], arrs[f"ut_{i}"] = u, ut
        arrs["checksums"] = np.array(sums)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        manifest[name] = dict(kind="wave_adapt_long", dim=dim, n_init=n0, nmax=nmax, eps=eps, eta=eta, sigma=sigma,
                              cfl=cfl, steps=steps, lagr_degree=4, snapshots=snaps, elements=elements)
        print(name, r["meta"], elements[-1])


# (name, dim, N, sigma, steps, dt): wave equation with interpolated K grad u, IPDG, RK4ODE2nd
WAVE_CASES = [
    ("wave2d_n4", 2, 4, 10.0, 2, 0.001),
    ("wave2d_n5", 2, 5, 10.0, 2, 0.0005),
    ("wave3d_n4", 3, 4, 20.0, 1, 0.0005),
]


# (name, dim, N_init, NMAX, eps, eta, sigma, cfl, steps): the adaptive wave loop
WAVE_ADAPT_CASES = [
    ("wave_adapt2d", 2, 3, 5, 1e-5, 1e-6, 10.0, 0.1, 4),
    ("wave_adapt3d", 3, 2, 4, 1e-3, 1e-4, 20.0, 0.05, 2),
]

# (name, dim, N_init, NMAX, eps, Lagrange degree, width): the adaptive-interpolation initialisation
# of exp(-width |x - (0.3, 0.4, 0.5)|^2)
INTP_CASES = [
    ("intp_init2d_m3", 2, 3, 6, 1e-4, 3, 100.0),
    ("intp_init2d_m4", 2, 3, 6, 1e-4, 4, 100.0),
    ("intp_init3d_m3", 3, 2, 5, 1e-3, 3, 50.0),
    ("intp_init2d_m5", 2, 3, 6, 1e-5, 5, 100.0),
    ("intp_init3d_m5", 3, 2, 5, 1e-4, 5, 50.0),
]


# (name, dim, N_init, NMAX, eps_a, eps_b, Lagrange degree, width): the split L2 error of one
# adaptive interpolation against a finer one
INTP_ERROR_CASES = [
    ("intp_error2d", 2, 3, 7, 1e-3, 1e-6, 3, 100.0),
    ("intp_error3d", 3, 2, 6, 1e-3, 1e-5, 4, 50.0),
]


def intp_cases(manifest):
    for name, dim, n0, nmax, ea, eb, degree, width in INTP_ERROR_CASES:
        r = run(["intp_error", dim, n0, nmax, repr(ea), repr(eb), degree, repr(width)])
        la, sa, ua = split_elements(r["u_a"], dim)
        lb, sb, ub = split_elements(r["u_b"], dim)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), level_a=la, suppt_a=sa, u_a=ua, level_b=lb,
                            suppt_b=sb, u_b=ub, err=r["err"].reshape(-1))
        manifest[name] = dict(kind="intp_error", dim=dim, n_init=n0, nmax=nmax, k=2, eps_a=ea, eps_b=eb,
                              lagr_degree=degree, width=width, centre=[0.3, 0.4, 0.5][:dim],
                              err=float(r["err"].reshape(-1)[0]))
        print(name, float(r["err"].reshape(-1)[0]), len(ua), len(ub))
    for name, dim, n0, nmax, eps, degree, width in INTP_CASES:
        r = run(["intp_init", dim, n0, nmax, repr(eps), degree, repr(width)])
        lv, sp, u = split_elements(r["u_init"], dim)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), level=lv, suppt=sp, u=u)
        manifest[name] = dict(kind="intp_init", dim=dim, n_init=n0, nmax=nmax, k=2, eps=eps, lagr_degree=degree,
                              width=width, centre=[0.3, 0.4, 0.5][:dim], elements=int(r["meta"]["elements"]))
        print(name, r["meta"])


def burgers_adapt_long(manifest):
    for name, dim, n0, nmax, eps, eta, alpha, cfl, umax, steps, snaps in BURGERS_ADAPT_LONG_CASES:
        res = subprocess.run([HARNESS, "burgers_adapt"] + [str(a) for a in (dim, n0, nmax, repr(eps), repr(eta),
                                                                             repr(alpha), repr(cfl), repr(umax), steps)],
                             check=True, capture_output=True, text=True)
        r = parse_harness(res.stdout)
        assert "HASH_OVERFLOW" not in res.stdout, "the reference's int32 element hash overflowed"
        maxlevsum = max(int(ln.split("maxlevsum=")[1].split()[0]) for ln in res.stdout.splitlines()
                        if ln.startswith("STEP"))
        dts = [float(ln.split("dt=")[1].split()[0]) for ln in res.stdout.splitlines() if ln.startswith("STEP")]
        arrs = {"dt": np.array(dts)}
        sums = []
        for i, key in enumerate(["u_init"] + [f"u_step{s}" for s in range(steps)]):
            lv, sp, u = split_elements(r[key], dim)
            arrs[f"level_{i}"], arrs[f"suppt_{i}"] = lv.astype(np.int16), sp.astype(np.int16)
            sums.append(checksums(lv, sp, u))
            if i in snaps:
                arrs[f"u_{i}"] = u
        arrs["checksums"] = np.array(sums)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        manifest[name] = dict(kind="burgers_adapt_long", dim=dim, n_init=n0, nmax=nmax, eps=eps, eta=eta,
                              alpha=alpha, cfl=cfl, umax=umax, steps=steps, snapshots=snaps,
                              max_level_sum=maxlevsum, t_end=float(np.sum(dts)),
                              elements=[int(len(arrs[f"level_{i}"])) for i in range(steps + 1)])
        print(name, r["meta"], "max level sum", maxlevsum)


# (name, N, alpha, steps, dt): 2D Burgers on the full sparse grid with the flux interpolated by
# cubic Hermite interpolation (HermInterpolation::nonlinear_Herm_2D_fast,
# HyperbolicSameFluxHermRHS, LxF penalty), SSP-RK3; u0 = 0.5 + 0.25 sin(2 pi (x+y))
HERM_CASES = [
    ("burgers_herm2d_n4", 4, 1.2, 2, 0.002),
    ("burgers_herm2d_n6", 6, 1.2, 1, 0.0005),
]

# (name, N_init, NMAX, eps, eta, alpha, cfl, steps, snapshot steps): the adaptive loop of
# example/02_hyperbolic_05_burgers_adapt.cpp (u0 = sin(2 pi (x+y)), Hermite flux, assembled LxF
# matrix, CFL 0.2 with wave speed 1): element sets and checksums after every step, coefficients at
# the snapshot steps (all of them when None)
HERM_ADAPT_CASES = [
    ("burgers_herm_adapt2d", 3, 6, 1e-4, 1e-5, 1.2, 0.2, 6, None),
    ("burgers_herm_adapt2d_n8_T003", 3, 8, 1e-5, 1e-6, 1.2, 0.2, 34, [0, 1, 2, 17, 34]),
]


def herm_cases(manifest):
    for name, N, alpha, steps, dt in HERM_CASES:
        r = run(["burgers_herm", N, repr(alpha), steps, repr(dt)])
        lv, sp, u0 = split_elements(r["u0"], 2)
        arrs = {"level": lv, "suppt": sp, "u0": u0}
        for key in ("up0", "fu0", "rhs0", "uT"):
            lv2, sp2, v = split_elements(r[key], 2)
            assert (lv == lv2).all() and (sp == sp2).all()
            arrs[key] = v
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        manifest[name] = dict(kind="burgers_herm", dim=2, N=N, k=2, herm_degree=3, alpha=alpha, steps=steps, dt=dt,
                              elements=int(r["meta"]["elements"]))
        print(name, r["meta"])
    for name, n0, nmax, eps, eta, alpha, cfl, steps, snaps in HERM_ADAPT_CASES:
        res = subprocess.run([HARNESS, "burgers_herm_adapt"] + [str(a) for a in (n0, nmax, repr(eps), repr(eta),
                                                                                  repr(alpha), repr(cfl), steps)],
                             check=True, capture_output=True, text=True)
        r = parse_harness(res.stdout)
        dts = [float(ln.split("dt=")[1].split()[0]) for ln in res.stdout.splitlines() if ln.startswith("STEP")]
        arrs, sums = {"dt": np.array(dts)}, []
        for i, key in enumerate(["u_init"] + [f"u_step{s}" for s in range(steps)]):
            lv, sp, u = split_elements(r[key], 2)
            arrs[f"level_{i}"], arrs[f"suppt_{i}"] = lv.astype(np.int16), sp.astype(np.int16)
            sums.append(checksums(lv, sp, u))
            if snaps is None or i in snaps:
                arrs[f"u_{i}"] = u
        arrs["checksums"] = np.array(sums)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        manifest[name] = dict(kind="burgers_herm_adapt", dim=2, n_init=n0, nmax=nmax, eps=eps, eta=eta, alpha=alpha,
                              cfl=cfl, steps=steps, snapshots=snaps, t_end=float(np.sum(dts)),
                              elements=[int(len(arrs[f"level_{i}"])) for i in range(steps + 1)])
        print(name, r["meta"], len(arrs[f"level_{steps}"]))


def main():
    if not os.path.exists(HARNESS):
        sys.exit("build the reference first: make -C oracle ref")
    only = {"intp": intp_cases, "burgers_adapt_long": burgers_adapt_long, "linear_long": linear_long,
            "wave_adapt_long": wave_adapt_long, "herm": herm_cases}
    if len(sys.argv) == 2 and sys.argv[1] in only:  # one group of cases, merged into the manifest
        path = os.path.join(HERE, "manifest.json")
        manifest = json.load(open(path))
        only[sys.argv[1]](manifest)
        with open(path, "w") as f:
            json.dump(manifest, f, indent=1)
        return
    manifest = {}
    for name, dim, N, k, ic, engine, steps, dt, c in LINEAR_CASES:
        r = run(["linear", dim, N, k, 1, ic, engine, steps, repr(dt)] + [repr(x) for x in c])
        lv, sp, u0 = split_elements(r["u0"], dim)
        lv2, sp2, rhs0 = split_elements(r["rhs0"], dim)
        lv3, sp3, uT = split_elements(r["uT"], dim)
        assert (lv == lv2).all() and (sp == sp2).all() and (lv == lv3).all() and (sp == sp3).all()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), level=lv, suppt=sp, u0=u0, rhs0=rhs0, uT=uT,
                            l2err=np.float64(r.get("l2err", np.nan)))
        manifest[name] = dict(kind="linear", dim=dim, N=N, k=k, ic=ic, engine=engine, steps=steps, dt=dt, c=c,
                              elements=int(r["meta"]["elements"]))
        print(name, r["meta"])
    for name, dim, N, alpha, steps, dt in BURGERS_CASES:
        r = run(["burgers", dim, N, repr(alpha), steps, repr(dt)])
        lv, sp, u0 = split_elements(r["u0"], dim)
        arrs = {"level": lv, "suppt": sp, "u0": u0}
        for key in ["up0", "rhs0", "uT"] + [f"fu0_{d}" for d in range(dim)]:
            lv2, sp2, v = split_elements(r[key], dim)
            assert (lv == lv2).all() and (sp == sp2).all()
            arrs[key] = v
        arrs["vals"] = r["vals"]
        for gp, err in r["normerr"].items():
            arrs[f"normerr_g{gp}"] = np.array(err)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        manifest[name] = dict(kind="burgers", dim=dim, N=N, k=2, alpha=alpha, steps=steps, dt=dt,
                              elements=int(r["meta"]["elements"]))
        print(name, r["meta"])
    for name, dim, n0, nmax, eps, eta, alpha, cfl, umax, steps in BURGERS_ADAPT_CASES:
        r = run(["burgers_adapt", dim, n0, nmax, repr(eps), repr(eta), repr(alpha), repr(cfl), repr(umax), steps])
        arrs = {}
        for i, key in enumerate(["u_init"] + [f"u_step{s}" for s in range(steps)]):
            lv, sp, u = split_elements(r[key], dim)
            arrs[f"level_{i}"], arrs[f"suppt_{i}"], arrs[f"u_{i}"] = lv, sp, u
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        manifest[name] = dict(kind="burgers_adapt", dim=dim, n_init=n0, nmax=nmax, eps=eps, eta=eta, alpha=alpha,
                              cfl=cfl, umax=umax, steps=steps)
        print(name, r["meta"])
    burgers_adapt_long(manifest)
    herm_cases(manifest)
    linear_long(manifest)
    for name, dim, N, sigma, steps, dt in WAVE_CASES:
        r = run(["wave", dim, N, repr(sigma), steps, repr(dt)])
        lv, sp, u0 = split_elements(r["u0"], dim)
        arrs = {"level": lv, "suppt": sp, "u0": u0}
        for key in ("rhs0", "uT", "vT"):
            lv2, sp2, v = split_elements(r[key], dim)
            idx = {tuple(a) + tuple(b): i for i, (a, b) in enumerate(zip(lv2, sp2))}
            arrs[key] = v[[idx[tuple(a) + tuple(b)] for a, b in zip(lv, sp)]]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        manifest[name] = dict(kind="wave", dim=dim, N=N, k=2, lagr_degree=4, sigma=sigma, steps=steps, dt=dt,
                              elements=int(r["meta"]["elements"]))
        print(name, r["meta"])
    for name, dim, n0, nmax, eps, eta, sigma, cfl, steps in WAVE_ADAPT_CASES:
        r = run(["wave_adapt", dim, n0, nmax, repr(eps), repr(eta), repr(sigma), repr(cfl), steps])
        arrs = {}
        for i, tag in enumerate(["init"] + [f"step{s}" for s in range(steps)]):
            lv, sp, u = split_elements(r["u_" + tag], dim)
            lv2, sp2, ut = split_elements(r["ut_" + tag], dim)
            assert (lv == lv2).all() and (sp == sp2).all()
            arrs[f"level_{i}"], arrs[f"suppt_{i}"], arrs[f"u_{i}"], arrs[f"ut_{i}"] = lv, sp, u, ut
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        manifest[name] = dict(kind="wave_adapt", dim=dim, n_init=n0, nmax=nmax, eps=eps, eta=eta, sigma=sigma,
                              cfl=cfl, steps=steps, lagr_degree=4)
        print(name, r["meta"])
    wave_adapt_long(manifest)
    intp_cases(manifest)
    for N, k in [(4, 2), (3, 1), (3, 3)]:
        r = run(["matrices", N, k])
        name = f"oper1d_n{N}_k{k}"
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            **{m: r[m] for m in ("u_v", "u_vx", "ulft_vjp", "urgt_vjp")})
        manifest[name] = dict(kind="oper1d", N=N, k=k)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
