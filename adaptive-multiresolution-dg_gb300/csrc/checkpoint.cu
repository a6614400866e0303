// Checkpoint / restart of a grid and the element-level dump of
// IO::output_element_level_support (IO.cpp:502-517).
//
// The reference has no checkpoint (its IO writes text tables only).  The file
// written here holds exactly what a restart needs, in the order the library
// keeps it:
//
//   offset  field
//   0       magic "AMDGCKP" followed by a zero byte
//   8       uint32 format version (1)
//   12      int32 dim, nmax, k, sparse
//   28      int32 flags (bit 0: the u_t field follows the coefficients)
//   32      int64 num_elements E
//   40      double time (the caller's, stored as given)
//   48      uint64 keys[E], ascending (packed 1D element orders, nmax bits per
//           dimension, first dimension most significant)
//           double u[E][(k+1)^dim]  (element-major, last dimension fastest)
//           double v[E][(k+1)^dim]  (when flags bit 0)
//   end-8   uint64 FNV-1a hash of every byte before it
//
// All fields are little-endian (both hosts the library builds for are).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "amdg.h"
#include "amdg_internal.hpp"

using namespace amdg;

namespace {

constexpr char kMagic[8] = {'A', 'M', 'D', 'G', 'C', 'K', 'P', '\0'};
constexpr uint32_t kVersion = 1;

struct Fnv {
    uint64_t h = 0xcbf29ce484222325ull;
    void add(const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) {
            h ^= b[i];
            h *= 0x100000001b3ull;
        }
    }
};

struct File {
    std::FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

bool write_all(std::FILE* f, Fnv* h, const void* p, size_t n) {
    h->add(p, n);
    return n == 0 || std::fwrite(p, 1, n, f) == n;
}

bool read_all(std::FILE* f, Fnv* h, void* p, size_t n) {
    if (n != 0 && std::fread(p, 1, n, f) != n) return false;
    h->add(p, n);
    return true;
}

amdg_status copy_from_device(const amdg_grid* g, const double* d, std::vector<double>* host) {
    host->resize(size_t(g->dof));
    cudaStream_t st = static_cast<cudaStream_t>(g->ctx->stream);
    cudaError_t e = cudaSuccess;
    if (g->dof) e = cudaMemcpyAsync(host->data(), d, size_t(g->dof) * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("checkpoint read-back: ") + cudaGetErrorString(e));
    return AMDG_OK;
}

// the support [xl, xr] of 1D element order o (Basis::supp_interv)
void support_of(int o, double* xl, double* xr) {
    int n, j;
    elem_of_order(o, &n, &j);
    if (n <= 1) {
        *xl = 0.0;
        *xr = 1.0;
        return;
    }
    const double h = std::pow(2.0, 1 - n);
    *xl = h * (j - 1) / 2.0;
    *xr = h * (j + 1) / 2.0;
}

}  // namespace

extern "C" {

amdg_status amdg_grid_save(const amdg_grid* g, const char* path, double time) {
    if (!g || !path) return fail(AMDG_ERR_ARG, "null argument");
    if (cudaSetDevice(g->device) != cudaSuccess) return fail(AMDG_ERR_CUDA, "cudaSetDevice failed");
    std::vector<double> u, v;
    amdg_status s = grid_ensure_host(g);
    if (s != AMDG_OK) return s;
    s = copy_from_device(g, g->d_u, &u);
    if (s != AMDG_OK) return s;
    const int32_t flags = g->d_v ? 1 : 0;
    if (flags && (s = copy_from_device(g, g->d_v, &v)) != AMDG_OK) return s;
    // write to a temporary name and rename, so a failed save leaves an earlier checkpoint intact
    const std::string tmp = std::string(path) + ".tmp";
    File out;
    out.f = std::fopen(tmp.c_str(), "wb");
    if (!out.f) return fail(AMDG_ERR_IO, "cannot open " + tmp + " for writing");
    Fnv h;
    const int32_t head[5] = {g->host.dim, g->host.nmax, g->host.k, g->host.sparse, flags};
    const int64_t E = g->host.num_elements;
    bool ok = write_all(out.f, &h, kMagic, sizeof kMagic) && write_all(out.f, &h, &kVersion, sizeof kVersion) &&
              write_all(out.f, &h, head, sizeof head) && write_all(out.f, &h, &E, sizeof E) &&
              write_all(out.f, &h, &time, sizeof time) &&
              write_all(out.f, &h, g->host.key.data(), g->host.key.size() * sizeof(uint64_t)) &&
              write_all(out.f, &h, u.data(), u.size() * sizeof(double)) &&
              (!flags || write_all(out.f, &h, v.data(), v.size() * sizeof(double)));
    const uint64_t sum = h.h;
    ok = ok && std::fwrite(&sum, 1, sizeof sum, out.f) == sizeof sum;
    ok = std::fclose(out.f) == 0 && ok;
    out.f = nullptr;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return fail(AMDG_ERR_IO, std::string("writing ") + path + " failed");
    }
    return AMDG_OK;
}

amdg_status amdg_grid_load(amdg_context* ctx, const char* path, amdg_grid** out, double* time) {
    if (!ctx || !path || !out) return fail(AMDG_ERR_ARG, "null argument");
    *out = nullptr;
    File in;
    in.f = std::fopen(path, "rb");
    if (!in.f) return fail(AMDG_ERR_IO, std::string("cannot open ") + path);
    Fnv h;
    char magic[8];
    uint32_t version = 0;
    int32_t head[5];
    int64_t E = 0;
    double t = 0.0;
    if (!read_all(in.f, &h, magic, sizeof magic) || std::memcmp(magic, kMagic, sizeof magic) != 0)
        return fail(AMDG_ERR_FORMAT, std::string(path) + " is not a grid checkpoint");
    if (!read_all(in.f, &h, &version, sizeof version) || version != kVersion)
        return fail(AMDG_ERR_FORMAT, std::string(path) + ": unsupported checkpoint version");
    if (!read_all(in.f, &h, head, sizeof head) || !read_all(in.f, &h, &E, sizeof E) || !read_all(in.f, &h, &t, sizeof t))
        return fail(AMDG_ERR_FORMAT, std::string(path) + ": truncated header");
    const int dim = head[0], nmax = head[1], k = head[2], sparse = head[3], flags = head[4];
    if (dim < 1 || dim > kMaxDim || k < 1 || k > 3 || nmax < 0 || nmax > 16 || dim * nmax > 60 || E < 1 ||
        E > (int64_t(1) << 31) - 1 || (flags & ~1) != 0)
        return fail(AMDG_ERR_FORMAT, std::string(path) + ": header out of range");
    int B = 1;
    for (int d = 0; d < dim; ++d) B *= k + 1;
    // the size the header implies must be the file's (before allocating anything from E)
    const long here = std::ftell(in.f);
    if (here < 0 || std::fseek(in.f, 0, SEEK_END) != 0) return fail(AMDG_ERR_IO, std::string("cannot seek in ") + path);
    const long end = std::ftell(in.f);
    const double want = double(here) + double(E) * 8.0 * (1.0 + double(B) * (1 + (flags & 1))) + 8.0;
    if (end < 0 || double(end) != want || std::fseek(in.f, here, SEEK_SET) != 0)
        return fail(AMDG_ERR_FORMAT, std::string(path) + ": file size does not match its header");
    std::vector<uint64_t> keys(size_t(E), 0);
    std::vector<double> u(size_t(E) * B), v(flags ? size_t(E) * B : 0);
    if (!read_all(in.f, &h, keys.data(), keys.size() * sizeof(uint64_t)) ||
        !read_all(in.f, &h, u.data(), u.size() * sizeof(double)) ||
        !read_all(in.f, &h, v.data(), v.size() * sizeof(double)))
        return fail(AMDG_ERR_FORMAT, std::string(path) + ": truncated");
    uint64_t sum = 0;
    if (std::fread(&sum, 1, sizeof sum, in.f) != sizeof sum || sum != h.h)
        return fail(AMDG_ERR_FORMAT, std::string(path) + ": checksum mismatch");
    // keys: strictly ascending, within dim * nmax bits (nmax bits per 1D order)
    for (size_t e = 0; e < keys.size(); ++e) {
        if (e > 0 && keys[e] <= keys[e - 1]) return fail(AMDG_ERR_FORMAT, std::string(path) + ": keys not ascending");
        if ((keys[e] >> (dim * nmax)) != 0) return fail(AMDG_ERR_FORMAT, std::string(path) + ": key out of range");
    }
    amdg_grid* g = nullptr;
    amdg_status s = amdg_grid_create_ex(ctx, dim, 0, nmax, k, sparse, &g);
    if (s != AMDG_OK) return s;
    if ((s = grid_set_keys(g, std::move(keys))) != AMDG_OK ||
        (s = amdg_grid_set_coefficients(g, u.data(), int64_t(u.size()))) != AMDG_OK ||
        (flags && (s = amdg_grid_set_velocity(g, v.data(), int64_t(v.size()))) != AMDG_OK)) {
        amdg_grid_destroy(g);
        return s;
    }
    if (time) *time = t;
    *out = g;
    return AMDG_OK;
}

amdg_status amdg_grid_config(const amdg_grid* g, int* dim, int* nmax, int* k, int* sparse) {
    if (!g) return fail(AMDG_ERR_ARG, "grid is null");
    if (dim) *dim = g->host.dim;
    if (nmax) *nmax = g->host.nmax;
    if (k) *k = g->host.k;
    if (sparse) *sparse = g->host.sparse;
    return AMDG_OK;
}

amdg_status amdg_grid_write_level_support(const amdg_grid* g, const char* path) {
    if (!g || !path) return fail(AMDG_ERR_ARG, "null argument");
    File out;
    out.f = std::fopen(path, "w");
    if (!out.f) return fail(AMDG_ERR_IO, std::string("cannot open ") + path + " for writing");
    if (amdg_status s = grid_ensure_host(g); s != AMDG_OK) return s;
    const int dim = g->host.dim;
    bool ok = true;
    for (int64_t e = 0; e < g->host.num_elements && ok; ++e) {
        for (int d = 0; d < dim && ok; ++d) {
            const int o = g->host.order[size_t(e) * dim + d];
            double xl, xr;
            support_of(o, &xl, &xr);
            ok = std::fprintf(out.f, "%d %g %g ", level_of_order(o), xl, xr) > 0;
        }
        ok = ok && std::fputc('\n', out.f) != EOF;
    }
    ok = std::fclose(out.f) == 0 && ok;
    out.f = nullptr;
    if (!ok) return fail(AMDG_ERR_IO, std::string("writing ") + path + " failed");
    return AMDG_OK;
}

}  // extern "C"
