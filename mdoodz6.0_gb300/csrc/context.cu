// Context lifetime, error reporting and host<->device marker transfers.
#include <algorithm>
#include <vector>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include "mdz_internal.cuh"

mdz_status mdz_fail(mdz_ctx *ctx, mdz_status s, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return s;
}

mdz_status mdz_cuda_check(mdz_ctx *ctx, cudaError_t e, const char *what) {
    return mdz_fail(ctx, MDZ_ERR_CUDA, "CUDA error in %s: %s", what, cudaGetErrorString(e));
}

void *mdz_stage(mdz_ctx *ctx, int slot, size_t bytes) {
    if (ctx->stage_bytes[slot] >= bytes && ctx->stage[slot]) return ctx->stage[slot];
    if (ctx->stage[slot]) cudaFree(ctx->stage[slot]);
    ctx->stage[slot] = nullptr;
    ctx->stage_bytes[slot] = 0;
    size_t b = bytes < 256 ? 256 : bytes;
    if (cudaMalloc(&ctx->stage[slot], b) != cudaSuccess) return nullptr;
    ctx->stage_bytes[slot] = b;
    return ctx->stage[slot];
}

mdz_nodeset mdz_get_nodeset(const mdz_ctx *ctx, int centroid) {
    const mdz_dgrid &g = ctx->g;
    mdz_nodeset s{};
    if (centroid == MDZ_NODES_CENTROIDS) { s.nx = g.Nx - 1; s.nz = g.Nz - 1; s.X = g.xc; s.Z = g.zc; s.tag = g.BCp; }
    else if (centroid == MDZ_NODES_VERTICES) { s.nx = g.Nx; s.nz = g.Nz; s.X = g.xg; s.Z = g.zg; s.tag = g.BCg; }
    else if (centroid == MDZ_NODES_VX) { s.nx = g.Nx; s.nz = g.Nz + 1; s.X = g.xg; s.Z = g.zvx; s.tag = g.BCu; }
    else { s.nx = g.Nx + 1; s.nz = g.Nz; s.X = g.xvz; s.Z = g.zg; s.tag = g.BCv; }
    return s;
}

template <typename T>
static cudaError_t upload(T **dst, const T *src, size_t n) {
    cudaError_t e = cudaMalloc((void **)dst, sizeof(T) * (n ? n : 1));
    if (e != cudaSuccess) return e;
    if (src && n) return cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice);
    return cudaMemset(*dst, 0, sizeof(T) * (n ? n : 1));
}

extern "C" mdz_status mdz_create(mdz_ctx **out, const mdz_grid_desc *d, int n_phases, long long max_markers) {
    if (!out || !d) return MDZ_ERR_ARG;
    *out = nullptr;
    mdz_ctx *ctx = new mdz_ctx();
    // (grids up to 65 535 lines a side: the marker kernels' index fast path,
    // ceil_quot, is exact up to quotients of 2^16)
    if (d->Nx < 3 || d->Nz < 3 || d->Nx > 65535 || d->Nz > 65535 || n_phases < 1 || n_phases > MDZ_MAX_PHASES ||
        max_markers < 0 || max_markers > (1LL << 31) - 1) {
        mdz_fail(ctx, MDZ_ERR_ARG, "mdz_create: bad grid size, phase count or marker capacity");
        delete ctx;
        return MDZ_ERR_ARG;
    }
    if (!d->xg || !d->zg || !d->xc || !d->zc || !d->xvz || !d->zvx || !d->BCu_type || !d->BCv_type ||
        !d->BCp_type || !d->BCg_type) {
        delete ctx;
        return MDZ_ERR_ARG;
    }
    if (d->isperiodic_x) {
        delete ctx;
        return MDZ_ERR_UNSUPPORTED;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        delete ctx;
        return MDZ_ERR_CUDA;
    }
    ctx->host_desc = *d;
    {
        const double *src[6] = {d->xg, d->zg, d->xc, d->zc, d->xvz, d->zvx};
        const size_t len[6] = {(size_t)d->Nx, (size_t)d->Nz, (size_t)d->Nx - 1, (size_t)d->Nz - 1,
                               (size_t)d->Nx + 1, (size_t)d->Nz + 1};
        for (int i = 0; i < 6; i++) ctx->hline[i].assign(src[i], src[i] + len[i]);
        const signed char *tsrc[4] = {d->BCu_type, d->BCv_type, d->BCp_type, d->BCg_type};
        const size_t tlen[4] = {(size_t)d->Nx * (d->Nz + 1), (size_t)(d->Nx + 1) * d->Nz,
                                (size_t)(d->Nx - 1) * (d->Nz - 1), (size_t)d->Nx * d->Nz};
        for (int i = 0; i < 4; i++) ctx->htag[i].assign(tsrc[i], tsrc[i] + tlen[i]);
        mdz_grid_desc &h = ctx->host_desc;
        h.xg = ctx->hline[0].data(); h.zg = ctx->hline[1].data(); h.xc = ctx->hline[2].data();
        h.zc = ctx->hline[3].data(); h.xvz = ctx->hline[4].data(); h.zvx = ctx->hline[5].data();
        h.BCu_type = ctx->htag[0].data(); h.BCv_type = ctx->htag[1].data();
        h.BCp_type = ctx->htag[2].data(); h.BCg_type = ctx->htag[3].data();
        h.BCu_val = nullptr; h.BCv_val = nullptr;
    }
    ctx->n_phases = n_phases;
    mdz_dgrid &g = ctx->g;
    int Nx = d->Nx, Nz = d->Nz;
    g.Nx = Nx; g.Nz = Nz; g.ncx = Nx - 1; g.ncz = Nz - 1;
    g.dx = d->dx; g.dz = d->dz;
    g.idx = 1.0 / d->dx; g.idz = 1.0 / d->dz;
    g.xmin = d->xmin; g.xmax = d->xmax; g.zmin = d->zmin; g.zmax = d->zmax;
    cudaError_t e = cudaSuccess;
#define UP(dst, src, n) if (e == cudaSuccess) e = upload(&dst, src, n)
    UP(g.xg, d->xg, Nx); UP(g.zg, d->zg, Nz); UP(g.xc, d->xc, Nx - 1); UP(g.zc, d->zc, Nz - 1);
    UP(g.xvz, d->xvz, Nx + 1); UP(g.zvx, d->zvx, Nz + 1);
    UP(g.BCu, d->BCu_type, (size_t)Nx * (Nz + 1)); UP(g.BCv, d->BCv_type, (size_t)(Nx + 1) * Nz);
    UP(g.BCp, d->BCp_type, (size_t)(Nx - 1) * (Nz - 1)); UP(g.BCg, d->BCg_type, (size_t)Nx * Nz);
    UP(g.BCu_val, d->BCu_val, (size_t)Nx * (Nz + 1)); UP(g.BCv_val, d->BCv_val, (size_t)(Nx + 1) * Nz);
    // markers
    long long cap = max_markers > 0 ? max_markers : 1;
    ctx->m.cap = max_markers;
    UP(ctx->m.x, (const double *)nullptr, cap); UP(ctx->m.z, (const double *)nullptr, cap);
    UP(ctx->m.vx, (const double *)nullptr, cap); UP(ctx->m.vz, (const double *)nullptr, cap);
    UP(ctx->m.phase, (const int *)nullptr, cap);
    for (int a = 0; a < MDZ_M_NATTR; a++) UP(ctx->m.attr[a], (const double *)nullptr, cap);
    int ncells = (Nx - 1) * (Nz - 1);
    ctx->bins.ncells = ncells;
    UP(ctx->bins.cell, (const int *)nullptr, cap); UP(ctx->bins.sorted, (const int *)nullptr, cap);
    UP(ctx->bins.qvert, (const int *)nullptr, cap);
    UP(ctx->bins.count, (const int *)nullptr, ncells + 1); UP(ctx->bins.start, (const int *)nullptr, ncells + 1);
    UP(ctx->bins.cursor, (const int *)nullptr, ncells + 1);
    UP(ctx->bins.scan_partials, (const int *)nullptr, (ncells + 1) / 1024 + 2);
    UP(ctx->red_part, (const double *)nullptr, MDZ_RED_PART);
    UP(ctx->red_cnt, (const unsigned int *)nullptr, MDZ_RED_COUNTERS);
#undef UP
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        mdz_destroy(ctx);
        return MDZ_ERR_CUDA;
    }
    *out = ctx;
    return MDZ_OK;
}

void mdz_free_fields(mdz_ctx *ctx);
void mdz_solver_free(mdz_ctx *ctx);
void mdz_mlp_free(mdz_ctx *ctx);

extern "C" void mdz_destroy(mdz_ctx *ctx) {
    if (!ctx) return;
    mdz_solver_free(ctx);
    mdz_mlp_free(ctx);
    mdz_reseed_free(ctx);
    mdz_free_fields(ctx);
    mdz_dgrid &g = ctx->g;
    void *ptrs[] = {g.xg, g.zg, g.xc, g.zc, g.xvz, g.zvx, g.BCu, g.BCv, g.BCp, g.BCg, g.BCu_val, g.BCv_val,
                    ctx->m.x, ctx->m.z, ctx->m.vx, ctx->m.vz, ctx->m.phase, ctx->bins.cell, ctx->bins.sorted,
                    ctx->bins.qvert, ctx->bins.count, ctx->bins.start, ctx->bins.cursor, ctx->bins.scan_partials,
                    ctx->red_part, ctx->red_cnt, ctx->ale_sums};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int a = 0; a < MDZ_M_NATTR; a++)
        if (ctx->m.attr[a]) cudaFree(ctx->m.attr[a]);
    for (int i = 0; i < 9; i++)
        if (ctx->stage[i]) cudaFree(ctx->stage[i]);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    for (cudaStream_t q : ctx->xfer)
        if (q) cudaStreamDestroy(q);
    delete ctx;
}

extern "C" const char *mdz_last_error(const mdz_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }
extern "C" long long mdz_kernel_launches(const mdz_ctx *ctx) { return ctx ? ctx->launches : 0; }
extern "C" int mdz_marker_count(const mdz_ctx *ctx) { return ctx ? ctx->m.n : 0; }

extern "C" mdz_status mdz_set_markers(mdz_ctx *ctx, int n, const double *x, const double *z, const int *phase) {
    if (!ctx) return MDZ_ERR_ARG;
    if (n < 0 || (n > 0 && (!x || !z || !phase))) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_set_markers: bad arguments");
    if (n > ctx->m.cap) return mdz_fail(ctx, MDZ_ERR_CAPACITY, "mdz_set_markers: %d markers > capacity %lld", n, ctx->m.cap);
    cudaStream_t st = ctx->stream;
    if (n) {
        MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->m.x, x, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->m.z, z, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->m.phase, phase, sizeof(int) * n, cudaMemcpyHostToDevice, st));
    }
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    ctx->m.n = n;
    ctx->bins.valid = false;
    return MDZ_OK;
}

extern "C" mdz_status mdz_set_marker_velocity(mdz_ctx *ctx, int n, const double *vx, const double *vz) {
    if (!ctx) return MDZ_ERR_ARG;
    if (n < 0 || n > ctx->m.n || (n > 0 && (!vx || !vz)))
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_set_marker_velocity: bad arguments (n=%d, resident %d)", n, ctx->m.n);
    cudaStream_t st = ctx->stream;
    if (n) {
        MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->m.vx, vx, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->m.vz, vz, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    }
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}

extern "C" mdz_status mdz_get_markers(mdz_ctx *ctx, int n, double *x, double *z, int *phase, double *vx, double *vz) {
    if (!ctx) return MDZ_ERR_ARG;
    if (n < 0 || n > ctx->m.n) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_get_markers: n=%d > resident %d", n, ctx->m.n);
    cudaStream_t st = ctx->stream;
    if (n) {
        if (x) MDZ_CUDA(ctx, cudaMemcpyAsync(x, ctx->m.x, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        if (z) MDZ_CUDA(ctx, cudaMemcpyAsync(z, ctx->m.z, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        if (phase) MDZ_CUDA(ctx, cudaMemcpyAsync(phase, ctx->m.phase, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
        if (vx) MDZ_CUDA(ctx, cudaMemcpyAsync(vx, ctx->m.vx, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        if (vz) MDZ_CUDA(ctx, cudaMemcpyAsync(vz, ctx->m.vz, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    }
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}

extern "C" mdz_status mdz_host_register(void *p, size_t bytes) {
    if (!p || bytes == 0) return MDZ_ERR_ARG;
    return cudaHostRegister(p, bytes, cudaHostRegisterDefault) == cudaSuccess ? MDZ_OK : MDZ_ERR_CUDA;
}

extern "C" mdz_status mdz_host_unregister(void *p) {
    if (!p) return MDZ_ERR_ARG;
    return cudaHostUnregister(p) == cudaSuccess ? MDZ_OK : MDZ_ERR_CUDA;
}

extern "C" mdz_status mdz_set_marker_attr(mdz_ctx *ctx, int attr, int n, const double *values) {
    if (!ctx) return MDZ_ERR_ARG;
    if (attr < 0 || attr >= MDZ_M_NATTR || n < 0 || n > ctx->m.n || (n > 0 && !values))
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_set_marker_attr: bad attribute %d or size %d (resident %d)", attr, n,
                        ctx->m.n);
    if (n) MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->m.attr[attr], values, sizeof(double) * n, cudaMemcpyHostToDevice,
                                         ctx->stream));
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MDZ_OK;
}

extern "C" mdz_status mdz_get_marker_attr(mdz_ctx *ctx, int attr, int n, double *values) {
    if (!ctx) return MDZ_ERR_ARG;
    if (attr < 0 || attr >= MDZ_M_NATTR || n < 0 || n > ctx->m.n || (n > 0 && !values))
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_get_marker_attr: bad attribute %d or size %d", attr, n);
    if (n) MDZ_CUDA(ctx, cudaMemcpyAsync(values, ctx->m.attr[attr], sizeof(double) * n, cudaMemcpyDeviceToHost,
                                         ctx->stream));
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MDZ_OK;
}

// ---- batched marker transfers ------------------------------------------------
// The reference's time loop keeps the markers in host arrays (x, z, phase and
// the attributes); a step through this library uploads them and reads the
// advected ones back.  One copy at a time on one stream moves 75-130 GB/s
// between the host and this GPU; the copies of one call are independent, so
// they are spread over MDZ_XFER_STREAMS streams (one cudaMemcpyAsync per
// array), ordered after the context's stream and joined back into it before
// the call returns.  Host arrays registered with mdz_host_register (or
// allocated pinned) make them DMA transfers.
struct xfer_copy {
    void *dst;
    const void *src;
    size_t bytes;
};

static mdz_status xfer_run(mdz_ctx *ctx, const xfer_copy *c, int nc, cudaMemcpyKind kind) {
    cudaStream_t st = ctx->stream;
    for (int q = 0; q < MDZ_XFER_STREAMS; q++)
        if (!ctx->xfer[q]) MDZ_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->xfer[q], cudaStreamNonBlocking));
    cudaEvent_t ready, done[MDZ_XFER_STREAMS];
    MDZ_CUDA(ctx, cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    MDZ_CUDA(ctx, cudaEventRecord(ready, st));
    for (int q = 0; q < MDZ_XFER_STREAMS; q++) {
        MDZ_CUDA(ctx, cudaEventCreateWithFlags(&done[q], cudaEventDisableTiming));
        MDZ_CUDA(ctx, cudaStreamWaitEvent(ctx->xfer[q], ready, 0));
    }
    // largest first, each to the stream with the fewest bytes so far
    std::vector<int> order(nc);
    for (int i = 0; i < nc; i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return c[a].bytes > c[b].bytes; });
    size_t load[MDZ_XFER_STREAMS] = {};
    for (int i : order) {
        if (!c[i].bytes) continue;
        int q = 0;
        for (int r = 1; r < MDZ_XFER_STREAMS; r++)
            if (load[r] < load[q]) q = r;
        load[q] += c[i].bytes;
        MDZ_CUDA(ctx, cudaMemcpyAsync(c[i].dst, c[i].src, c[i].bytes, kind, ctx->xfer[q]));
    }
    for (int q = 0; q < MDZ_XFER_STREAMS; q++) {
        MDZ_CUDA(ctx, cudaEventRecord(done[q], ctx->xfer[q]));
        MDZ_CUDA(ctx, cudaStreamWaitEvent(st, done[q], 0));
    }
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    cudaEventDestroy(ready);
    for (int q = 0; q < MDZ_XFER_STREAMS; q++) cudaEventDestroy(done[q]);
    return MDZ_OK;
}

extern "C" mdz_status mdz_set_marker_state(mdz_ctx *ctx, int n, const double *x, const double *z, const int *phase,
                                           const double *const *attrs) {
    if (!ctx) return MDZ_ERR_ARG;
    if (n < 0 || (n > 0 && (!x || !z || !phase)))
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_set_marker_state: bad arguments");
    if (n > ctx->m.cap)
        return mdz_fail(ctx, MDZ_ERR_CAPACITY, "mdz_set_marker_state: %d markers > capacity %lld", n, ctx->m.cap);
    xfer_copy c[3 + MDZ_M_NATTR];
    int nc = 0;
    const size_t b8 = sizeof(double) * (size_t)n;
    c[nc++] = {ctx->m.x, x, b8};
    c[nc++] = {ctx->m.z, z, b8};
    c[nc++] = {ctx->m.phase, phase, sizeof(int) * (size_t)n};
    for (int a = 0; attrs && a < MDZ_M_NATTR; a++)
        if (attrs[a]) c[nc++] = {ctx->m.attr[a], attrs[a], b8};
    mdz_status s = xfer_run(ctx, c, nc, cudaMemcpyHostToDevice);
    if (s != MDZ_OK) return s;
    ctx->m.n = n;
    ctx->bins.valid = false;
    return MDZ_OK;
}

extern "C" mdz_status mdz_get_marker_state(mdz_ctx *ctx, int n, double *x, double *z, int *phase, double *vx,
                                           double *vz, double *const *attrs) {
    if (!ctx) return MDZ_ERR_ARG;
    if (n < 0 || n > ctx->m.n)
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_get_marker_state: n=%d > resident %d", n, ctx->m.n);
    xfer_copy c[5 + MDZ_M_NATTR];
    int nc = 0;
    const size_t b8 = sizeof(double) * (size_t)n;
    if (x) c[nc++] = {x, ctx->m.x, b8};
    if (z) c[nc++] = {z, ctx->m.z, b8};
    if (phase) c[nc++] = {phase, ctx->m.phase, sizeof(int) * (size_t)n};
    if (vx) c[nc++] = {vx, ctx->m.vx, b8};
    if (vz) c[nc++] = {vz, ctx->m.vz, b8};
    for (int a = 0; attrs && a < MDZ_M_NATTR; a++)
        if (attrs[a]) c[nc++] = {attrs[a], ctx->m.attr[a], b8};
    return xfer_run(ctx, c, nc, cudaMemcpyDeviceToHost);
}

// ---- optional launch timing of the main kernel classes -------------------------
void mdz_prof_begin(mdz_ctx *ctx, int cls, cudaStream_t st, cudaEvent_t *ev) {
    (void)cls;
    *ev = nullptr;
    if (!ctx->profiling) return;
    cudaEventCreate(ev);
    cudaEventRecord(*ev, st);
}

void mdz_prof_end(mdz_ctx *ctx, int cls, double bytes, cudaStream_t st, cudaEvent_t a) {
    if (!ctx->profiling || !a) return;
    cudaEvent_t b;
    cudaEventCreate(&b);
    cudaEventRecord(b, st);
    ctx->prof.push_back(mdz_ctx::prof_rec{cls, a, b, bytes});
}

static void prof_resolve(mdz_ctx *ctx) {
    for (auto &r : ctx->prof) {
        cudaEventSynchronize(r.b);
        float ms = 0;
        cudaEventElapsedTime(&ms, r.a, r.b);
        ctx->prof_ms[r.cls] += ms;
        ctx->prof_bytes[r.cls] += r.bytes;
        ctx->prof_n[r.cls] += 1;
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    ctx->prof.clear();
}

extern "C" mdz_status mdz_set_profiling(mdz_ctx *ctx, int on) {
    if (!ctx) return MDZ_ERR_ARG;
    prof_resolve(ctx);
    for (int i = 0; i < 8; i++) { ctx->prof_ms[i] = 0; ctx->prof_bytes[i] = 0; ctx->prof_n[i] = 0; }
    ctx->profiling = on != 0;
    return MDZ_OK;
}

extern "C" mdz_status mdz_kernel_timing(mdz_ctx *ctx, int cls, double *ms, double *bytes, long long *launches) {
    if (!ctx || cls < 0 || cls >= MDZ_PROF_NCLS) return MDZ_ERR_ARG;
    prof_resolve(ctx);
    if (ms) *ms = ctx->prof_ms[cls];
    if (bytes) *bytes = ctx->prof_bytes[cls];
    if (launches) *launches = ctx->prof_n[cls];
    return MDZ_OK;
}

extern "C" mdz_status mdz_sync(mdz_ctx *ctx) {
    if (!ctx) return MDZ_ERR_ARG;
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MDZ_OK;
}
