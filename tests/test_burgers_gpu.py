"""Parity of the CUDA Lagrange-interpolation path (Burgers flux, LxF) with the
reference fixtures and the oracle.  Tolerances: FP64 1e-12 relative to the
field's max norm for point values, flux coefficients and RK3 steps, 5e-12 for
one RHS (a difference of larger volume and interface terms); mixed mode
(FP64 point values and surplus, FP32 back transforms and penalty, FP64
state) 1e-4 relative in the L2 norm for one RHS (FP32 rounding of back
transforms whose 1D matrices grow like 2^level) and 1e-6 for RK3 steps."""
import numpy as np
import pytest

import amdg
import amdg_oracle as O
from helpers import align, golden, manifest, rel_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

BURGERS = [n for n, m in manifest().items() if m["kind"] == "burgers"]


def dev(n):
    return torch.zeros(n, dtype=torch.float64, device="cuda")


def run_on(ctx, fn, u, nout):
    """Copy u to the device, call fn(d_u, d_out), return the output on the host."""
    torch.cuda.synchronize()
    du = torch.from_numpy(np.ascontiguousarray(u).reshape(-1)).cuda()
    out = dev(nout)
    torch.cuda.synchronize()
    fn(du.data_ptr(), out.data_ptr())
    ctx.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("name", BURGERS)
def test_burgers_matches_reference(ctx, name):
    m = manifest()[name]
    z = golden(name)
    dim, N, k = m["dim"], m["N"], m["k"]
    g = amdg.Grid(ctx, dim, N, k)
    lv, sp = g.elements()
    perm = align(z["level"], z["suppt"], lv, sp)
    g.init_separable(O.burgers_ic_terms(dim))
    assert rel_err(g.coefficients(), z["u0"][perm]) < 1e-13
    u0 = np.ascontiguousarray(z["u0"][perm])
    op = amdg.BurgersOperator(g, m["alpha"])
    P = 4 ** dim
    up = run_on(ctx, op.point_values_device, u0, g.num_elements * P).reshape(-1, P)
    assert rel_err(up, z["up0"][perm]) < 1e-12
    fu = run_on(ctx, op.flux_coefficients_device, u0, g.num_elements * P).reshape(-1, P)
    assert rel_err(fu, z["fu0_0"][perm]) < 1e-12
    rhs = run_on(ctx, op.rhs_device, u0, g.dof).reshape(-1, g.block)
    assert rel_err(rhs, z["rhs0"][perm]) < 5e-12
    rhs32 = run_on(ctx, lambda a, b: op.rhs_device(a, b, amdg.MIXED), u0, g.dof).reshape(-1, g.block)
    ref = z["rhs0"][perm]
    assert np.linalg.norm(rhs32 - ref) / np.linalg.norm(ref) < 1e-4
    g.set_coefficients(u0)
    op.rk3_steps(m["dt"], m["steps"], amdg.FP64)
    ctx.synchronize()
    assert rel_err(g.coefficients(), z["uT"][perm]) < 1e-12
    g.set_coefficients(u0)
    op.rk3_steps(m["dt"], m["steps"], amdg.MIXED)
    ctx.synchronize()
    assert rel_err(g.coefficients(), z["uT"][perm]) < 1e-6
    op.close()
    g.close()


def test_burgers_3d_n6_matches_oracle(ctx):
    dim, N, k, alpha = 3, 6, 2, 0.825
    g = amdg.Grid(ctx, dim, N, k)
    lv, sp = g.elements()
    g.init_separable(O.burgers_ic_terms(dim))
    u0 = g.coefficients().copy()
    op = amdg.BurgersOperator(g, alpha)
    rhs = run_on(ctx, op.rhs_device, u0, g.dof).reshape(-1, g.block)
    ref, _, _ = O.burgers_rhs(dim, N, k, lv, sp, u0, alpha)
    assert rel_err(rhs, ref) < 5e-12
    op.close()
    g.close()


def test_burgers_rhs_deterministic_and_hole_detection(ctx):
    g = amdg.Grid(ctx, 2, 5, 2)
    g.init_separable(O.burgers_ic_terms(2))
    u0 = g.coefficients().copy()
    op = amdg.BurgersOperator(g, 1.0)
    a = run_on(ctx, op.rhs_device, u0, g.dof)
    b = run_on(ctx, op.rhs_device, u0, g.dof)
    assert np.array_equal(a, b)
    op.close()
    g.close()


@pytest.mark.parametrize("prec", [amdg.FP64, amdg.MIXED])
def test_rhs_term_groups_add_up_to_the_fused_rhs(ctx, prec):
    """LagrInterpolation + rhs_vol_scalar + rhs_flx_intp_scalar + rhs_flx_penalty_scalar called one
    by one into the grid's rhs equal the fused right-hand side bitwise (same terms, same order)."""
    dim, N = 3, 4
    g = amdg.Grid(ctx, dim, N, 2)
    g.init_separable(O.burgers_ic_terms(dim))
    op = amdg.BurgersOperator(g, 0.825)
    du = torch.from_numpy(g.coefficients().reshape(-1).copy()).cuda()
    fused = torch.zeros_like(du)
    torch.cuda.synchronize()
    op.rhs_device(du.data_ptr(), fused.data_ptr(), prec)
    op.interpolate(prec)
    g.set_rhs_zero()
    for group in (op.RHS_VOL, op.RHS_FLX, op.RHS_PENALTY):
        op.rhs_add(group, 0.825 if group == op.RHS_PENALTY else None, prec=prec)
    assert np.array_equal(g.rhs().reshape(-1), fused.cpu().numpy())
    # the penalty constant of the call replaces the operator's
    g.set_rhs_zero()
    op.rhs_add(op.RHS_PENALTY, 1.5, prec=prec)
    pen15 = g.rhs().copy()
    g.set_rhs_zero()
    op.rhs_add(op.RHS_PENALTY, 0.75, prec=prec)
    assert np.allclose(pen15, 2.0 * g.rhs(), rtol=1e-12, atol=0)
    op.close()
    g.close()


@pytest.mark.parametrize("prec", [amdg.FP64, amdg.MIXED])
def test_sweep_variants_agree_bitwise(ctx, prec):
    """The two transform-sweep kernels (thread per output entry, thread per column) sum every
    output in the same order: identical right-hand sides, on a sparse and an adaptive grid."""
    for dim, N, adaptive in ((3, 5, False), (2, 7, True)):
        g = amdg.Grid(ctx, dim, N, 2, level_init=3 if adaptive else None)
        if adaptive:
            g.init_separable_adaptive(O.burgers_ic_terms(dim), 1e-4)
        else:
            g.init_separable(O.burgers_ic_terms(dim))
        op = amdg.BurgersOperator(g, 0.825)
        du = torch.from_numpy(g.coefficients().reshape(-1).copy()).cuda()
        outs = []
        for variant in (0, 1):
            op.set_sweep_variant(variant)
            out = torch.zeros_like(du)
            torch.cuda.synchronize()
            op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
            ctx.synchronize()
            outs.append(out.cpu().numpy())
        assert np.array_equal(outs[0], outs[1])
        op.close()
        g.close()


@pytest.mark.parametrize("prec,tol", [(amdg.FP64, 1e-12), (amdg.MIXED, 1e-4)])
def test_warp_sweep_variant_matches(ctx, prec, tol):
    """The warp-per-(term, element) sweep kernel sums in another fixed order: its right-hand sides
    equal the thread-per-output kernel's to rounding (relative to the field's max; mixed: FP32
    back transforms of a right-hand side that is a difference of large flux terms, the 1e-4 of the
    mixed right-hand-side bar), are
    deterministic run to run, and in FP64 match the oracle to 5e-12 on the 3D sparse grid N = 6 and
    the 2D wave grid (degree-4 points, 5 -> 3 and 3 -> 5 transforms)."""
    cases = [("burgers", 3, 6, False), ("burgers", 2, 7, True), ("wave", 2, 6, False)]
    for kind, dim, N, adaptive in cases:
        g = amdg.Grid(ctx, dim, N, 2, level_init=3 if adaptive else None)
        if kind == "wave":
            g.init_separable(O.wave_ic_terms(dim))
            op = amdg.WaveOperator(g, 10.0)
        elif adaptive:
            g.init_separable_adaptive(O.burgers_ic_terms(dim), 1e-4)
            op = amdg.BurgersOperator(g, 0.825)
        else:
            g.init_separable(O.burgers_ic_terms(dim))
            op = amdg.BurgersOperator(g, 0.825)
        u = g.coefficients().copy()
        du = torch.from_numpy(u.reshape(-1).copy()).cuda()
        outs = []
        for variant in (0, 2, 2):
            op.set_sweep_variant(variant)
            out = torch.zeros_like(du)
            torch.cuda.synchronize()
            op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
            ctx.synchronize()
            outs.append(out.cpu().numpy())
        scale = np.abs(outs[0]).max()
        assert np.abs(outs[1] - outs[0]).max() <= tol * scale, (kind, dim, N)
        assert np.array_equal(outs[1], outs[2])
        if prec == amdg.FP64 and not adaptive:
            lv, sp = g.elements()
            if kind == "wave":
                ref = O.wave_rhs(dim, N, 2, lv, sp, u, 10.0)
            else:
                ref = O.burgers_rhs(dim, N, 2, lv, sp, u, 0.825)[0]
            assert np.abs(outs[1].reshape(ref.shape) - ref).max() <= 5e-12 * np.abs(ref).max()
        op.close()
        g.close()
