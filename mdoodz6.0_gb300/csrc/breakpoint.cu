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

// Host arrays of a restarted state into the device mirrors: n markers (x, z,
// vx, vz, phase and the MDZ_M_NATTR attribute arrays), u, v, p (or nullptr:
// a state saved before any field existed, whose fields were zero) and the box.
mdz_status install_state(mdz_ctx *ctx, int n, const double *const xzv[4], const int *phase,
                         const double *const attr[MDZ_M_NATTR], const double *u, const double *v, const double *p,
                         const double box[4]) {
    const mdz_dgrid &g = ctx->g;
    const size_t nu = (size_t)g.Nx * (g.Nz + 1), nv = (size_t)(g.Nx + 1) * g.Nz, np = (size_t)g.ncx * g.ncz;
    if (u) {
        mdz_status s = mdz_ensure_fields(ctx);
        if (s != MDZ_OK) return s;
    }
    double *dst[4] = {ctx->m.x, ctx->m.z, ctx->m.vx, ctx->m.vz};
    if (n) {
        for (int i = 0; i < 4; i++)
            MDZ_CUDA(ctx, cudaMemcpy(dst[i], xzv[i], sizeof(double) * n, cudaMemcpyHostToDevice));
        MDZ_CUDA(ctx, cudaMemcpy(ctx->m.phase, phase, sizeof(int) * n, cudaMemcpyHostToDevice));
        for (int a = 0; a < MDZ_M_NATTR; a++)
            MDZ_CUDA(ctx, cudaMemcpy(ctx->m.attr[a], attr[a], sizeof(double) * n, cudaMemcpyHostToDevice));
    }
    if (u) {
        MDZ_CUDA(ctx, cudaMemcpy(ctx->d.u, u, sizeof(double) * nu, cudaMemcpyHostToDevice));
        MDZ_CUDA(ctx, cudaMemcpy(ctx->d.v, v, sizeof(double) * nv, cudaMemcpyHostToDevice));
        MDZ_CUDA(ctx, cudaMemcpy(ctx->d.p, p, sizeof(double) * np, cudaMemcpyHostToDevice));
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
    if (box[0] != d.xmin || box[1] != d.xmax || box[2] != d.zmin || box[3] != d.zmax)
        return mdz_set_box(ctx, box[0], box[1], box[2], box[3], ctx->stream);
    return MDZ_OK;
}
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
    const double *xzv[4], *attr[MDZ_M_NATTR];
    for (int a = 0; a < 4; a++) xzv[a] = mk.data() + (size_t)a * n;
    for (int a = 0; a < MDZ_M_NATTR; a++) attr[a] = mk.data() + (size_t)(4 + a) * n;
    const double box[4] = {h.xmin, h.xmax, h.zmin, h.zmax};
    return install_state(ctx, n, xzv, ph.data(), attr, h.has_fields ? fl.data() : nullptr,
                         h.has_fields ? fl.data() + nu : nullptr, h.has_fields ? fl.data() + nu + nv : nullptr, box);
}

// Restart from the reference's own breakpoint (Breakpoint%05d.dat, written by
// MakeBreakpointParticles, SOURCE/InputOutput.c:515-903): the file is read as
// LoadBreakpointParticles (:160-514) reads it -- a 4-byte size header (int,
// double, DoodzFP, char), dt, dt0, time and the box, the topography chains
// when free_surf, Nb_part and the marker arrays, the grid arrays of the
// previous step, u_in / v_in / p_in, then topography, boundary tags and
// values, phase proportions and marker counts -- with the sections that the
// run's flags switch on.  What this library keeps is taken (positions,
// velocities, phases, P, the deviatoric stresses when iselastic, strain,
// plastic strain, T, and u_in, v_in, p_in as the step's starting u, v, p),
// divided by the run's scales as the reference's loader divides them; the
// rest is rebuilt by the next step.  The file length must be exactly the
// length those flags give for this grid and phase count, so a wrong flag, a
// file of another grid or a truncated file is refused before anything changes.
extern "C" mdz_status mdz_load_reference_breakpoint(mdz_ctx *ctx, const char *path,
                                                    const mdz_ref_breakpoint_desc *desc, double *dt,
                                                    double *time) {
    if (!ctx) return MDZ_ERR_ARG;
    if (!path || !desc) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_reference_breakpoint: null argument");
    if (!(desc->L > 0) || !(desc->V > 0) || !(desc->S > 0) || !(desc->T > 0) || !(desc->t > 0))
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_reference_breakpoint: the scales must be positive");
    const mdz_dgrid &g = ctx->g;
    const size_t Nx = (size_t)g.Nx, nc = (size_t)g.ncx * g.ncz, ns = Nx * g.Nz, nu = Nx * (g.Nz + 1),
                 nv = (Nx + 1) * g.Nz;
    file_closer fc{fopen(path, "rb")};
    if (!fc.f) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_reference_breakpoint: cannot open %s", path);
    std::vector<unsigned char> buf;
    {
        unsigned char chunk[1 << 16];
        size_t got;
        while ((got = fread(chunk, 1, sizeof chunk, fc.f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    }
    size_t pos = 0;
    bool ok = true;
    auto take = [&](void *dst, size_t bytes) {
        if (!ok || bytes > buf.size() - pos) {
            ok = false;
            return;
        }
        if (dst) memcpy(dst, buf.data() + pos, bytes);
        pos += bytes;
    };
    unsigned char sizes[4] = {0, 0, 0, 0};
    take(sizes, 4);
    if (!ok || sizes[0] != 4 || sizes[1] != 8 || sizes[2] != 8 || sizes[3] != 1)
        return mdz_fail(ctx, MDZ_ERR_ARG,
                        "mdz_load_reference_breakpoint: %s is not a breakpoint of 4-byte int, 8-byte double and DoodzFP",
                        path);
    double hdr[7];   // dt, dt0, time, xmin, xmax, zmin, zmax
    take(hdr, sizeof hdr);
    if (desc->free_surf)
        for (int c = 0; c < 2 && ok; c++) {   // topography chain and its initial copy: Nb_part, x, z, Vx, Vz
            int nb = -1;
            take(&nb, 4);
            if (nb < 0) ok = false;
            take(nullptr, 4 * 8 * (size_t)(nb < 0 ? 0 : nb));
        }
    int n = -1;
    take(&n, 4);
    if (!ok || n < 0)
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_reference_breakpoint: %s is truncated before the markers", path);
    if (n > ctx->m.cap)
        return mdz_fail(ctx, MDZ_ERR_CAPACITY, "mdz_load_reference_breakpoint: %d markers > capacity %lld", n,
                        ctx->m.cap);
    const size_t dn = 8 * (size_t)n;
    std::vector<double> xzv[4], attr[MDZ_M_NATTR];
    for (auto &a : xzv) a.assign(n, 0.0);
    for (auto &a : attr) a.assign(n, 0.0);
    std::vector<int> ph(n);
    take(xzv[0].data(), dn);                   // x
    take(xzv[1].data(), dn);                   // z
    take(attr[MDZ_M_P].data(), dn);            // P
    take(xzv[2].data(), dn);                   // Vx
    take(xzv[3].data(), dn);                   // Vz
    take(nullptr, 2 * dn);                     // phi, X
    take(ph.data(), 4 * (size_t)n);            // phase
    if (desc->iselastic) {
        take(attr[MDZ_M_SXXD].data(), dn);
        take(attr[MDZ_M_SZZD].data(), dn);
        take(attr[MDZ_M_SXZ].data(), dn);
        take(nullptr, 3 * dn);                 // dsxxd, dszzd, dsxz
        take(nullptr, 8 * (2 * nc + 2 * ns));  // eta_n, VE_n, eta_s, VE_s
    }
    take(attr[MDZ_M_STRAIN].data(), dn);
    take(nullptr, dn);                         // strain_el
    take(attr[MDZ_M_STRAIN_PL].data(), dn);
    take(nullptr, 5 * dn);                     // strain_pwl, strain_exp, strain_lin, strain_gbs, d
    if (desc->fstrain) take(nullptr, 4 * dn);
    if (desc->aniso) take(nullptr, 4 * dn);
    if (desc->rec_T_P_x_z) take(nullptr, 6 * dn);
    take(nullptr, dn);                         // divth
    take(attr[MDZ_M_T].data(), dn);
    take(nullptr, dn);                         // rho
    take(nullptr, 8 * (9 * nc + (desc->aniso ? 2 * nc : 0)));   // p0_n ... szzd0, nx0_n, nz0_n
    take(nullptr, 8 * (2 * ns + (desc->aniso ? 2 * ns : 0)));   // X0_s, sxz0, nx0_s, nz0_s
    take(nullptr, 8 * (nc + ns));              // eta_phys_n, eta_phys_s
    std::vector<double> u(nu), v(nv), p(nc);
    take(u.data(), 8 * nu);
    take(v.data(), 8 * nv);
    take(p.data(), 8 * nc);
    // what follows: p_lith, p_lith0, Ut, W, L0, the two topographies, the
    // boundary tags (char) and values, the phase proportions and the counts
    const size_t topo = desc->free_surf ? 2 * 8 * (4 * Nx + 1 + 4 * (Nx - 1)) : 0;
    const size_t rest = 8 * (2 * nc + 3) + topo + (2 * nc + nu + nv + ns) + 8 * (nc + nu + nv + ns) +
                        8 * (size_t)ctx->n_phases * (nc + ns) + 4 * (nc + ns);
    if (!ok || buf.size() - pos != rest)
        return mdz_fail(ctx, MDZ_ERR_ARG,
                        "mdz_load_reference_breakpoint: %s (%zu bytes) does not have the layout of a breakpoint of this "
                        "%dx%d grid with %d phases and these flags",
                        path, buf.size(), g.Nx, g.Nz, ctx->n_phases);
    for (int k = 0; k < n; k++)
        if (ph[k] < -1 || ph[k] >= ctx->n_phases)
            return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_reference_breakpoint: marker %d has phase %d", k, ph[k]);
    // back to the scaled units, as the reference's loader does
    for (int k = 0; k < n; k++) {
        xzv[0][k] /= desc->L;
        xzv[1][k] /= desc->L;
        xzv[2][k] /= desc->V;
        xzv[3][k] /= desc->V;
        attr[MDZ_M_P][k] /= desc->S;
        if (desc->iselastic) {
            attr[MDZ_M_SXXD][k] /= desc->S;
            attr[MDZ_M_SZZD][k] /= desc->S;
            attr[MDZ_M_SXZ][k] /= desc->S;
        }
        attr[MDZ_M_T][k] /= desc->T;
        attr[MDZ_M_CMUL][k] = 1.0;   // no reference marker array: 1 is the reference's own cohesion
    }
    for (auto &w : u) w /= desc->V;
    for (auto &w : v) w /= desc->V;
    for (auto &w : p) w /= desc->S;
    const double box[4] = {hdr[3] / desc->L, hdr[4] / desc->L, hdr[5] / desc->L, hdr[6] / desc->L};
    if (!(box[1] > box[0]) || !(box[3] > box[2]))
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_load_reference_breakpoint: %s holds an empty box", path);
    const double *xp[4] = {xzv[0].data(), xzv[1].data(), xzv[2].data(), xzv[3].data()}, *ap[MDZ_M_NATTR];
    for (int a = 0; a < MDZ_M_NATTR; a++) ap[a] = attr[a].data();
    mdz_status s = install_state(ctx, n, xp, ph.data(), ap, u.data(), v.data(), p.data(), box);
    if (s != MDZ_OK) return s;
    if (dt) *dt = hdr[0] / desc->t;
    if (time) *time = hdr[2] / desc->t;
    return MDZ_OK;
}
