// Breakpoint of the resident state: the counterpart of MakeBreakpointParticles
// / LoadBreakpointParticles (SOURCE/InputOutput.c:515-1007, 160-514) for what this library keeps
// on the device between time steps.  The reference dumps its host arrays;
// here the markers (positions, phases, velocities, the MDZ_M_* attributes) and
// the grid velocity and pressure that start the next step go from the device
// mirrors to one binary file and back, so that a restarted run continues as
// the uninterrupted one.  Everything else a step needs is rebuilt from these
// (projections, rheology, multigrid hierarchy); the learned guess's weights
// have their own entry points (mdz_mlp_get_weights / mdz_mlp_set_weights).
//
// File: "MDZBRK02", int32 Nx, Nz, n_phases, n_markers, n_attr, has_fields,
// double xmin, xmax, zmin, zmax (the box, which PureShearALE moves), then x,
// z, vx, vz (double), phase (int32), the n_attr attribute arrays (double) and,
// when has_fields, u, v, p (double), in the byte order of the host that wrote
// it.  Loading restores the box and regenerates the grid lines over it, as
// the reference reads model.xmin..zmax back and calls SetGridCoordinates
// (Main_DOODZ.c:446).
#include <cstdio>
#include <cstring>
#include <vector>
#include "mdz_internal.cuh"

namespace {
const char kMagic[8] = {'M', 'D', 'Z', 'B', 'R', 'K', '0', '2'};

struct brk_header {
    char magic[8];
    int Nx, Nz, n_phases, n_markers, n_attr, has_fields;
    double xmin, xmax, zmin, zmax;
};

struct file_closer {
    FILE *f;
    ~file_closer() { if (f) fclose(f); }
};
}  // namespace

extern "C" mdz_status mdz_save_breakpoint(mdz_ctx *ctx, const char *path) {
    if (!ctx) return MDZ_ERR_ARG;
    if (!path) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_save_breakpoint: null path");
    const mdz_dgrid &g = ctx->g;
    const int n = ctx->m.n;
    const size_t nu = (size_t)g.Nx * (g.Nz + 1), nv = (size_t)(g.Nx + 1) * g.Nz, np = (size_t)g.ncx * g.ncz;
    brk_header h;
    memcpy(h.magic, kMagic, 8);
    h.Nx = g.Nx; h.Nz = g.Nz; h.n_phases = ctx->n_phases; h.n_markers = n; h.n_attr = MDZ_M_NATTR;
    h.has_fields = ctx->fields_ready ? 1 : 0;
    h.xmin = ctx->host_desc.xmin; h.xmax = ctx->host_desc.xmax;
    h.zmin = ctx->host_desc.zmin; h.zmax = ctx->host_desc.zmax;
    // one host staging buffer, filled array by array from the device
    const size_t big = (size_t)n > nu + nv + np ? (size_t)n : nu + nv + np;
    std::vector<double> buf(big > 0 ? big : 1);
    std::vector<int> ibuf(n > 0 ? n : 1);
    file_closer fc{fopen(path, "wb")};
    if (!fc.f) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_save_breakpoint: cannot open %s", path);
    cudaStream_t st = ctx->stream;
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    bool ok = fwrite(&h, sizeof h, 1, fc.f) == 1;
    auto put = [&](const double *d, size_t cnt) -> mdz_status {
        if (cnt == 0) return MDZ_OK;
        MDZ_CUDA(ctx, cudaMemcpy(buf.data(), d, sizeof(double) * cnt, cudaMemcpyDeviceToHost));
        ok = ok && fwrite(buf.data(), sizeof(double), cnt, fc.f) == cnt;
        return MDZ_OK;
    };
    mdz_status s;
    const double *mk[4] = {ctx->m.x, ctx->m.z, ctx->m.vx, ctx->m.vz};
    for (const double *d : mk)
        if ((s = put(d, (size_t)n)) != MDZ_OK) return s;
    if (n) {
        MDZ_CUDA(ctx, cudaMemcpy(ibuf.data(), ctx->m.phase, sizeof(int) * n, cudaMemcpyDeviceToHost));
        ok = ok && fwrite(ibuf.data(), sizeof(int), (size_t)n, fc.f) == (size_t)n;
    }
    for (int a = 0; a < MDZ_M_NATTR; a++)
        if ((s = put(ctx->m.attr[a], (size_t)n)) != MDZ_OK) return s;
    if (h.has_fields) {
        if ((s = put(ctx->d.u, nu)) != MDZ_OK) return s;
        if ((s = put(ctx->d.v, nv)) != MDZ_OK) return s;
        if ((s = put(ctx->d.p, np)) != MDZ_OK) return s;
    }
    if (!ok) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_save_breakpoint: write to %s failed", path);
    return MDZ_OK;
}

extern "C" mdz_status mdz_load_breakpoint(mdz_ctx *ctx, const char *path) {
    if (!ctx) return MDZ_ERR_ARG;
    if (!path) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_breakpoint: null path");
    const mdz_dgrid &g = ctx->g;
    file_closer fc{fopen(path, "rb")};
    if (!fc.f) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_breakpoint: cannot open %s", path);
    brk_header h;
    if (fread(&h, sizeof h, 1, fc.f) != 1 || memcmp(h.magic, kMagic, 8) != 0)
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_breakpoint: %s is not a breakpoint of this library", path);
    if (h.Nx != g.Nx || h.Nz != g.Nz || h.n_phases != ctx->n_phases || h.n_attr != MDZ_M_NATTR ||
        !(h.xmax > h.xmin) || !(h.zmax > h.zmin))
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_breakpoint: %s holds another grid (%dx%d, %d phases)", path, h.Nx,
                        h.Nz, h.n_phases);
    if (h.n_markers < 0 || h.n_markers > ctx->m.cap)
        return mdz_fail(ctx, MDZ_ERR_CAPACITY, "mdz_load_breakpoint: %d markers > capacity %lld", h.n_markers,
                        ctx->m.cap);
    const int n = h.n_markers;
    const size_t nu = (size_t)g.Nx * (g.Nz + 1), nv = (size_t)(g.Nx + 1) * g.Nz, np = (size_t)g.ncx * g.ncz;
    // read everything before touching the device: a short file changes nothing
    std::vector<double> mk((size_t)(4 + MDZ_M_NATTR) * n), fl(h.has_fields ? nu + nv + np : 0);
    std::vector<int> ph(n);
    bool ok = fread(mk.data(), sizeof(double), 4 * (size_t)n, fc.f) == 4 * (size_t)n;
    ok = ok && fread(ph.data(), sizeof(int), (size_t)n, fc.f) == (size_t)n;
    ok = ok && fread(mk.data() + 4 * (size_t)n, sizeof(double), (size_t)MDZ_M_NATTR * n, fc.f) ==
                   (size_t)MDZ_M_NATTR * n;
    if (h.has_fields) ok = ok && fread(fl.data(), sizeof(double), fl.size(), fc.f) == fl.size();
    if (!ok) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_breakpoint: %s is truncated", path);
    if (h.has_fields) {
        mdz_status s = mdz_ensure_fields(ctx);
        if (s != MDZ_OK) return s;
    }
    double *dst[4] = {ctx->m.x, ctx->m.z, ctx->m.vx, ctx->m.vz};
    if (n) {
        for (int i = 0; i < 4; i++)
            MDZ_CUDA(ctx, cudaMemcpy(dst[i], mk.data() + (size_t)i * n, sizeof(double) * n, cudaMemcpyHostToDevice));
        MDZ_CUDA(ctx, cudaMemcpy(ctx->m.phase, ph.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
        for (int a = 0; a < MDZ_M_NATTR; a++)
            MDZ_CUDA(ctx, cudaMemcpy(ctx->m.attr[a], mk.data() + (size_t)(4 + a) * n, sizeof(double) * n,
                                     cudaMemcpyHostToDevice));
    }
    if (h.has_fields) {
        MDZ_CUDA(ctx, cudaMemcpy(ctx->d.u, fl.data(), sizeof(double) * nu, cudaMemcpyHostToDevice));
        MDZ_CUDA(ctx, cudaMemcpy(ctx->d.v, fl.data() + nu, sizeof(double) * nv, cudaMemcpyHostToDevice));
        MDZ_CUDA(ctx, cudaMemcpy(ctx->d.p, fl.data() + nu + nv, sizeof(double) * np, cudaMemcpyHostToDevice));
    } else if (ctx->fields_ready) {
        // saved before any field existed: the saving context's u, v, p were
        // zero, so a context that has stepped since must not keep its own
        MDZ_CUDA(ctx, cudaMemset(ctx->d.u, 0, sizeof(double) * nu));
        MDZ_CUDA(ctx, cudaMemset(ctx->d.v, 0, sizeof(double) * nv));
        MDZ_CUDA(ctx, cudaMemset(ctx->d.p, 0, sizeof(double) * np));
    }
    ctx->m.n = n;
    ctx->bins.valid = false;
    const mdz_grid_desc &d = ctx->host_desc;
    if (h.xmin != d.xmin || h.xmax != d.xmax || h.zmin != d.zmin || h.zmax != d.zmax)
        return mdz_set_box(ctx, h.xmin, h.xmax, h.zmin, h.zmax, ctx->stream);
    return MDZ_OK;
}
