// Many independent simulations advanced together (sm_103a).
//
// The reference runs one simulation per Solver; for many small ones every
// stage would be a handful of tiny launches.  A batch concatenates the
// instances' particles into one particle set and gives every instance its
// own dense grid (cell size from its own smoothing length), fixed at set-up
// with a margin, so that a whole time step -- neighbour build, density +
// Tait + neighbour lists, rates, FP64 update -- is a fixed sequence of
// launches over all instances with no host synchronisation and no
// allocation.  That sequence is captured once into a CUDA graph and
// replayed.  Particles that leave their instance's grid or jump more than
// one reference cell set bits of a device error word instead of stopping
// the step; sph_batch_error_word reports them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sph_internal.cuh"

namespace sphgb {

namespace {

constexpr int kThreads = 256;

__global__ void k_inst_fill(int *inst_of, int64_t offset, int64_t n, int k) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        inst_of[offset + i] = k;
}

// keys on the per-instance grids (+ jump check against the instance's
// reference cell, base/cell.pyx:1422-1437)
__global__ void k_bkeys(sph_array_view a, const Grid *grids, const double *inv_cs_ref,
                        const int *inst_of, int *key, int *count, int *refcell, int check_jump,
                        unsigned *err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int k = inst_of[i];
        const Grid &g = grids[k];
        const double p[3] = {ld0(a.x, i), ld0(a.y, i), ld0(a.z, i)};
        int c[3];
        const int b0[3] = {g.bx0, g.by0, g.bz0};
        const int nn[3] = {g.nx, g.ny, g.nz};
        const int kk[3] = {g.kx, g.ky, g.kz};
        bool out = false;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int v = (int)floor(p[d] * g.inv_cs) - b0[d];
            // the stencil of a cell reaches k cells beyond it: keep k of margin
            if (v < kk[d] || v >= nn[d] - kk[d]) {
                out = true;
                v = min(max(v, kk[d]), nn[d] - 1 - kk[d]);
            }
            c[d] = v;
        }
        if (out) atomicOr(err, SPH_EFLAG_BOX);
        const int kc = (int)g.cell_base + c[0] + g.nx * (c[1] + g.ny * c[2]);
        key[i] = kc;
        atomicAdd(&count[kc], 1);
        const double ir = inv_cs_ref[k];
        bool jump = false;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int rc = (int)floor(p[d] * ir);
            if (check_jump && abs(rc - refcell[3 * i + d]) > 1) jump = true;
            refcell[3 * i + d] = rc;
        }
        if (jump) atomicOr(err, SPH_EFLAG_JUMP);
    }
}

__global__ void k_breorder(sph_array_view a, const Grid *grids, const int *inst_of,
                           const int *perm, const int *key, int *skey, int *sinst, float *scx,
                           float4 *velh, float4 *st, float4 *pm) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < a.n;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int i = perm[s];
        const int k = inst_of[i];
        const Grid &g = grids[k];
        const int kl = key[i] - (int)g.cell_base;
        skey[s] = kl;
        sinst[s] = k;
        int cx, cy, cz;
        decode_cell(g, kl, cx, cy, cz);
        const double ox = (double)(cx + g.bx0), oy = (double)(cy + g.by0), oz = (double)(cz + g.bz0);
        const float xi = (float)fma(-ox, g.cs, ld0(a.x, i)), yi = (float)fma(-oy, g.cs, ld0(a.y, i)),
                    zi = (float)fma(-oz, g.cs, ld0(a.z, i));
        scx[s] = (float)cx;
        velh[s] = make_float4((float)ld0(a.u, i), (float)ld0(a.v, i), (float)ld0(a.w, i),
                              (float)a.h[i]);
        const float rho = (float)ld0(a.rho, i), p = (float)ld0(a.p, i), m = (float)a.m[i];
        st[s] = make_float4(rho, p / (rho * rho), (float)ld0(a.cs, i), m);
        pm[s] = make_float4(xi, yi, zi, m);
    }
}

// Bounding box of every instance's current positions (instance k owns the
// original indices [off[k], off[k + 1])), one block per instance.
__global__ void k_inst_box(sph_array_view a, const int64_t *off, double *box) {
    const int k = blockIdx.x;
    const int64_t i0 = off[k], i1 = off[k + 1];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const double p[3] = {ld0(a.x, i), ld0(a.y, i), ld0(a.z, i)};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], p[d]);
            hi[d] = fmax(hi[d], p[d]);
        }
    }
    __shared__ double red[6][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
        if (lane == 0) {
            red[d][wid] = lo[d];
            red[3 + d][wid] = hi[d];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int q = threadIdx.x;
        double v = red[q][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            v = q < 3 ? fmin(v, red[q][w]) : fmax(v, red[q][w]);
        box[6 * k + q] = v;
    }
}

// Count of the steps that completed (a step whose launches were gated off
// by the error word is not counted).
__global__ void k_step_done(const unsigned *err, unsigned long long *steps) {
    if (*err == 0u) *steps += 1ull;
}

}  // namespace

// Lay out the per-instance grids over the regions [lo, hi] (3 doubles per
// instance each): cell size from the instance's own reference cell and
// subdivision, the cells of the instances of subdivision 1, then 2, then 3
// one after another in the shared cell table (so the sorted slots come in
// the same groups), the cell table (re)allocated when it grows.
int batch_place(sph_batch *b, const double *lo, const double *hi) {
    const int ninst = b->ninst;
    b->h_grids.assign(ninst, Grid());
    b->groups.clear();
    int64_t cells = 0, slot = 0;
    for (int K = 1; K <= 3; ++K) {
        BatchGroup grp;
        grp.K = K;
        grp.s0 = slot;
        for (int k = 0; k < ninst; ++k) {
            if (b->inst_subdiv[k] != K) continue;
            Grid &g = b->h_grids[k];
            const double *l = lo + 3 * k, *h = hi + 3 * k;
            g.cs = b->inst_cell[k] / K;
            g.inv_cs = 1.0 / g.cs;
            g.cs_f = (float)g.cs;
            g.radius_scale = b->rec.radius_scale;
            g.kx = K;
            g.ky = (h[1] > l[1]) ? K : 0;
            g.kz = (h[2] > l[2]) ? K : 0;
            int c0[3], c1[3];
            for (int d = 0; d < 3; ++d) {
                c0[d] = (int)std::floor(l[d] * g.inv_cs);
                c1[d] = (int)std::floor(h[d] * g.inv_cs);
            }
            g.bx0 = c0[0] - g.kx;
            g.by0 = c0[1] - g.ky;
            g.bz0 = c0[2] - g.kz;
            const int64_t nx = (int64_t)c1[0] - c0[0] + 1 + 2 * g.kx;
            const int64_t ny = (int64_t)c1[1] - c0[1] + 1 + 2 * g.ky;
            const int64_t nz = (int64_t)c1[2] - c0[2] + 1 + 2 * g.kz;
            if (nx * ny * nz > ((int64_t)1 << 26) || nx > (1 << 24))
                return set_error(SPH_ERR_GRID, "batch: an instance's region needs too many cells");
            g.nx = (int)nx; g.ny = (int)ny; g.nz = (int)nz;
            g.ncells = nx * ny * nz;
            g.cell_base = cells;
            g.uniform_h = b->h_uniform_inst[k];
            cells += g.ncells;
            slot += b->inst_off[k + 1] - b->inst_off[k];
        }
        grp.s1 = slot;
        if (grp.s1 > grp.s0) b->groups.push_back(grp);
    }
    if (cells >= ((int64_t)1 << 30)) return set_error(SPH_ERR_GRID, "batch: too many cells in total");
    b->total_cells = cells;
    cudaStream_t st = b->stream;
    ArraySnap &A = b->snap;
    if (cells + 1 > b->cell_cap) {
        cudaFree(A.cstart);
        cudaFree(A.cursor);
        A.cstart = A.cursor = nullptr;
        const int64_t cap = cells + 1 + (cells + 1) / 4;
        SPH_CUDA(cudaMalloc(&A.cstart, sizeof(int) * cap));
        SPH_CUDA(cudaMalloc(&A.cursor, sizeof(int) * cap));
        b->cell_cap = cap;
        // scan scratch (sized now: nothing is allocated while a step is captured)
        const int64_t ntiles = (cap + 2047) / 2048 + 1;
        if (ntiles > b->ctx->scan_tmp_cap) {
            cudaFree(b->ctx->scan_tmp);
            b->ctx->scan_tmp = nullptr;
            SPH_CUDA(cudaMalloc(&b->ctx->scan_tmp, sizeof(int) * ntiles));
            b->ctx->scan_tmp_cap = ntiles;
        }
    }
    SPH_CUDA(cudaMemcpyAsync(b->d_grids, b->h_grids.data(), sizeof(Grid) * ninst,
                             cudaMemcpyHostToDevice, st));
    // the host vector must outlive the copy
    SPH_CUDA(cudaStreamSynchronize(st));
    return SPH_OK;
}

// New regions from the instances' current extents (grown by the margin),
// the grids laid out again and the step graph dropped (re-captured at the
// next step).
int batch_regrid(sph_batch *b) {
    cudaStream_t st = b->stream;
    const int ninst = b->ninst;
    k_inst_box<<<ninst, 256, 0, st>>>(b->view, b->d_off, b->d_ibox);
    count_launch();
    SPH_LAUNCH_CHECK("k_inst_box");
    std::vector<double> box(6 * (size_t)ninst), lo(3 * (size_t)ninst), hi(3 * (size_t)ninst);
    SPH_CUDA(cudaMemcpyAsync(box.data(), b->d_ibox, sizeof(double) * box.size(),
                             cudaMemcpyDeviceToHost, st));
    SPH_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < ninst; ++k)
        for (int d = 0; d < 3; ++d) {
            const double l = box[6 * k + d], h = box[6 * k + 3 + d];
            const double ext = h - l;
            const double pad = ext > 0 ? b->margin * ext + 4.0 * b->inst_cell[k] : 0.0;
            lo[3 * k + d] = l - pad;
            hi[3 * k + d] = h + pad;
        }
    const int rc = batch_place(b, lo.data(), hi.data());
    if (rc) return rc;
    if (b->graph_exec) {
        cudaGraphExecDestroy(b->graph_exec);
        b->graph_exec = nullptr;
    }
    b->regrids += 1;
    return SPH_OK;
}

int batch_build(sph_batch *b, int check_jump) {
    cudaStream_t st = b->stream;
    const int64_t n = b->view.n;
    ArraySnap &A = b->snap;
    SPH_CUDA(cudaMemsetAsync(A.cstart, 0, sizeof(int) * (b->total_cells + 1), st));
    const int nb = grid_blocks(n, kThreads);
    k_bkeys<<<nb, kThreads, 0, st>>>(b->view, b->d_grids, b->d_inv_ref, b->inst_of, A.key,
                                     A.cstart, A.refcell, check_jump && b->steps_built > 0,
                                     b->d_err);
    count_launch();
    SPH_LAUNCH_CHECK("k_bkeys");
    int rc = scan_exclusive(b->ctx, A.cstart, b->total_cells + 1);
    if (rc) return rc;
    SPH_CUDA(cudaMemcpyAsync(A.cursor, A.cstart, sizeof(int) * b->total_cells,
                             cudaMemcpyDeviceToDevice, st));
    launch_counting_sort(st, n, b->total_cells, A.key, A.cursor, A.cstart, A.perm);
    k_breorder<<<nb, kThreads, 0, st>>>(b->view, b->d_grids, b->inst_of, A.perm, A.key, A.skey,
                                        b->sinst, A.scx, A.velh, A.st, A.pm);
    count_launch();
    SPH_LAUNCH_CHECK("k_breorder");
    b->steps_built += 1;
    return SPH_OK;
}

int batch_setup(sph_batch *b, const sph_array_view *all, const sph_batch_instance *inst,
                int ninst, const sph_batch_recipe *rec) {
    if (!all || !inst || ninst <= 0 || !rec) return set_error(SPH_ERR_ARG, "batch: null argument");
    if (all->n <= 0 || !all->x || !all->h || !all->m || !all->rho || !all->p || !all->cs)
        return set_error(SPH_ERR_ARG, "batch: particle arrays need x, h, m, rho, p, cs");
    if (rec->subdiv < 1 || rec->subdiv > 3) return set_error(SPH_ERR_ARG, "batch: subdiv must be 1..3");
    if (rec->scheme != 0 && rec->scheme != 1) return set_error(SPH_ERR_ARG, "batch: scheme 0 (Euler) or 1 (RK2)");
    if (rec->dim < 1 || rec->dim > 3) return set_error(SPH_ERR_ARG, "batch: dim must be 1..3");
    if (rec->density.h0 != 0.0)
        return set_error(SPH_ERR_NOTSUP, "batch: the density pass runs at the particles' own h");
    if (rec->term.flags & SPH_TERM_VDIV)
        return set_error(SPH_ERR_NOTSUP, "batch: no velocity divergence term");
    int64_t covered = 0;
    for (int k = 0; k < ninst; ++k) {
        if (inst[k].offset != covered || inst[k].n <= 0)
            return set_error(SPH_ERR_ARG, "batch: instances must tile [0, n) in order");
        if (!(inst[k].cell_size > 0)) return set_error(SPH_ERR_ARG, "batch: cell_size must be > 0");
        covered += inst[k].n;
    }
    if (covered != all->n) return set_error(SPH_ERR_ARG, "batch: instances must cover every particle");
    if (all->n >= (int64_t)1 << 23) return set_error(SPH_ERR_NOTSUP, "batch: at most 2^23 particles");
    b->view = *all;
    b->rec = *rec;
    b->ninst = ninst;
    b->margin = rec->margin > 0 ? rec->margin : 0.0;
    b->inst_subdiv.assign(ninst, rec->subdiv);
    b->inst_cell.assign(ninst, 0.0);
    b->h_uniform_inst.assign(ninst, 0);
    b->inst_off.assign(ninst + 1, 0);
    std::vector<double> lo(3 * (size_t)ninst), hi(3 * (size_t)ninst);
    for (int k = 0; k < ninst; ++k) {
        if (inst[k].subdiv < 0 || inst[k].subdiv > 3)
            return set_error(SPH_ERR_ARG, "batch: an instance's subdiv must be 0..3");
        if (inst[k].subdiv > 0) b->inst_subdiv[k] = inst[k].subdiv;
        b->inst_cell[k] = inst[k].cell_size;
        b->h_uniform_inst[k] = inst[k].uniform_h ? 1 : 0;
        b->inst_off[k + 1] = inst[k].offset + inst[k].n;
        for (int d = 0; d < 3; ++d) {
            lo[3 * k + d] = inst[k].lo[d];
            hi[3 * k + d] = inst[k].hi[d];
        }
    }
    b->uniform_h = 1;
    for (int k = 0; k < ninst; ++k) b->uniform_h &= b->h_uniform_inst[k];
    cudaStream_t st = b->stream;
    const int64_t n = all->n;
    std::vector<double> inv_ref(ninst);
    for (int k = 0; k < ninst; ++k) inv_ref[k] = 1.0 / inst[k].cell_size;
    SPH_CUDA(cudaMalloc(&b->d_grids, sizeof(Grid) * ninst));
    SPH_CUDA(cudaMalloc(&b->d_inv_ref, sizeof(double) * ninst));
    SPH_CUDA(cudaMemcpyAsync(b->d_inv_ref, inv_ref.data(), sizeof(double) * ninst,
                             cudaMemcpyHostToDevice, st));
    SPH_CUDA(cudaMalloc(&b->d_off, sizeof(int64_t) * (ninst + 1)));
    SPH_CUDA(cudaMemcpyAsync(b->d_off, b->inst_off.data(), sizeof(int64_t) * (ninst + 1),
                             cudaMemcpyHostToDevice, st));
    SPH_CUDA(cudaMalloc(&b->d_ibox, sizeof(double) * 6 * ninst));
    SPH_CUDA(cudaMalloc(&b->d_steps, sizeof(unsigned long long)));
    SPH_CUDA(cudaMemsetAsync(b->d_steps, 0, sizeof(unsigned long long), st));
    b->h_steps = 0;
    {
        const int rc = batch_place(b, lo.data(), hi.data());
        if (rc) return rc;
    }
    SPH_CUDA(cudaMalloc(&b->inst_of, sizeof(int) * n));
    SPH_CUDA(cudaMalloc(&b->sinst, sizeof(int) * n));
    for (int k = 0; k < ninst; ++k) {
        k_inst_fill<<<grid_blocks(inst[k].n, kThreads), kThreads, 0, st>>>(b->inst_of, inst[k].offset,
                                                                          inst[k].n, k);
        count_launch();
    }
    ArraySnap &A = b->snap;
    A.n = n;
    SPH_CUDA(cudaMalloc(&A.key, sizeof(int) * n));
    SPH_CUDA(cudaMalloc(&A.perm, sizeof(int) * n));
    SPH_CUDA(cudaMalloc(&A.skey, sizeof(int) * n));
    SPH_CUDA(cudaMalloc(&A.scx, sizeof(float) * n));
    SPH_CUDA(cudaMalloc(&A.pm, sizeof(float4) * n));
    SPH_CUDA(cudaMalloc(&A.velh, sizeof(float4) * n));
    SPH_CUDA(cudaMalloc(&A.st, sizeof(float4) * n));
    SPH_CUDA(cudaMalloc(&A.refcell, sizeof(int) * 3 * n));
    A.view = *all;
    // neighbour list (built by every first density pass)
    NbrList &L = b->list;
    L.cap = rec->list_cap > 0 ? rec->list_cap : (rec->dim == 3 ? 96 : (rec->dim == 2 ? 40 : 16));
    L.stride = n;
    SPH_CUDA(cudaMalloc(&L.nbr, sizeof(uint32_t) * n * L.cap));
    SPH_CUDA(cudaMalloc(&L.cnt, sizeof(int) * n));
    SPH_CUDA(cudaMalloc(&L.maxcnt, sizeof(int)));
    SPH_CUDA(cudaMemsetAsync(L.maxcnt, 0, sizeof(int), st));
    L.entries = n * L.cap;
    // integrator work arrays: per integrated component, x0 (RK2), rate1, rate2
    const int ncomp = rec->dim;
    for (int c = 0; c < 2 * ncomp; ++c) {
        SPH_CUDA(cudaMalloc(&b->rate1[c], sizeof(double) * n));
        SPH_CUDA(cudaMalloc(&b->rate2[c], sizeof(double) * n));
        SPH_CUDA(cudaMalloc(&b->x0[c], sizeof(double) * n));
    }
    SPH_CUDA(cudaMalloc(&b->d_err, sizeof(unsigned)));
    SPH_CUDA(cudaMemsetAsync(b->d_err, 0, sizeof(unsigned), st));
    SPH_CUDA(cudaStreamSynchronize(st));
    b->ready = true;
    return SPH_OK;
}

// one evaluation: neighbour build, density (+Tait, +lists), rates
static int batch_eval(sph_batch *b, double *const *rate) {
    int rc = batch_build(b, 1);
    if (rc) return rc;
    rc = batch_density(b);
    if (rc) return rc;
    double *acc[3] = {nullptr, nullptr, nullptr}, *pos[3] = {nullptr, nullptr, nullptr};
    for (int c = 0; c < b->rec.dim; ++c) {
        pos[c] = rate[c];
        acc[c] = rate[b->rec.dim + c];
    }
    return batch_rates(b, acc, pos);
}

// state pointers of integrated component c: x, y, z then u, v, w
static double *state_ptr(sph_batch *b, int c) {
    const int d = b->rec.dim;
    const double *p[6] = {b->view.x, b->view.y, b->view.z, b->view.u, b->view.v, b->view.w};
    return const_cast<double *>(p[c < d ? c : 3 + (c - d)]);
}

// one time step as a fixed launch sequence (captured into the graph); every
// launch that writes the state, and the completed-step count, is gated on
// the error word, so a step in which a particle left its region or jumped
// changes nothing after that point
static int batch_step_launches_gated(sph_batch *b);

static int batch_step_launches(sph_batch *b) {
    b->ctx->gate = b->d_err;
    const int rc = batch_step_launches_gated(b);
    b->ctx->gate = nullptr;
    if (rc) return rc;
    k_step_done<<<1, 1, 0, b->stream>>>(b->d_err, b->d_steps);
    count_launch();
    SPH_LAUNCH_CHECK("k_step_done");
    return SPH_OK;
}

static int batch_step_launches_gated(sph_batch *b) {
    const int nc = 2 * b->rec.dim;
    const double dt = b->rec.dt;
    sph_axpy_line lines[SPH_MAX_AXPY_LINES];
    int rc;
    if (b->rec.scheme == 0) {
        rc = batch_eval(b, b->rate1);
        if (rc) return rc;
        for (int c = 0; c < nc; ++c)
            lines[c] = sph_axpy_line{state_ptr(b, c), nullptr, state_ptr(b, c), b->rate1[c], nullptr, dt, 1};
        return launch_integrate(b->ctx, b->view.n, lines, nc);
    }
    for (int c = 0; c < nc; ++c)
        lines[c] = sph_axpy_line{b->x0[c], nullptr, state_ptr(b, c), nullptr, nullptr, 0.0, 2};
    rc = launch_integrate(b->ctx, b->view.n, lines, nc);
    if (rc) return rc;
    rc = batch_eval(b, b->rate1);
    if (rc) return rc;
    for (int c = 0; c < nc; ++c)
        lines[c] = sph_axpy_line{state_ptr(b, c), nullptr, b->x0[c], b->rate1[c], nullptr, dt, 1};
    rc = launch_integrate(b->ctx, b->view.n, lines, nc);
    if (rc) return rc;
    rc = batch_eval(b, b->rate2);
    if (rc) return rc;
    for (int c = 0; c < nc; ++c)
        lines[c] = sph_axpy_line{state_ptr(b, c), nullptr, b->x0[c], b->rate1[c], b->rate2[c],
                                 0.5 * dt, 0};
    return launch_integrate(b->ctx, b->view.n, lines, nc);
}

// Launch nsteps steps: replays of the captured step graph, or eager
// launches.
static int batch_launch_steps(sph_batch *b, int nsteps, int use_graph) {
    if (!use_graph) {
        for (int s = 0; s < nsteps; ++s) {
            const int rc = batch_step_launches(b);
            if (rc) return rc;
        }
        return SPH_OK;
    }
    if (!b->graph_exec) {
        // the first build of a batch fills the jump reference; run one step
        // outside the graph so every captured build can check jumps
        if (b->steps_built == 0) {
            const int rc = batch_step_launches(b);
            if (rc) return rc;
            --nsteps;
        }
        cudaGraph_t graph = nullptr;
        SPH_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = batch_step_launches(b);
        cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cuda_check(e, "cudaStreamEndCapture");
        // kernels per replay, for the launch counter (the captured launches
        // were counted at capture but did not run then)
        size_t nnodes = 0;
        e = cudaGraphGetNodes(graph, nullptr, &nnodes);
        std::vector<cudaGraphNode_t> nodes(nnodes);
        if (e == cudaSuccess && nnodes) e = cudaGraphGetNodes(graph, nodes.data(), &nnodes);
        int kernels = 0;
        for (size_t i = 0; e == cudaSuccess && i < nnodes; ++i) {
            cudaGraphNodeType t;
            e = cudaGraphNodeGetType(nodes[i], &t);
            kernels += (e == cudaSuccess && t == cudaGraphNodeTypeKernel);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_check(e, "cudaGraphInstantiate");
        b->graph_kernels = kernels;
        count_launch(-kernels);
    }
    for (int s = 0; s < nsteps; ++s) {
        SPH_CUDA(cudaGraphLaunch(b->graph_exec, b->stream));
        count_launch(b->graph_kernels);
    }
    return SPH_OK;
}

int batch_step(sph_batch *b, int nsteps, int use_graph) {
    if (!b->ready) return set_error(SPH_ERR_STATE, "batch: not set up");
    if (nsteps < 0) return set_error(SPH_ERR_ARG, "batch: negative step count");
    int left = nsteps, stuck = 0;
    while (left > 0) {
        int rc = batch_launch_steps(b, left, use_graph);
        if (rc) return rc;
        // the steps completed and the error word
        struct {
            unsigned long long steps;
            unsigned err;
        } h{0, 0};
        SPH_CUDA(cudaMemcpyAsync(&h.steps, b->d_steps, sizeof(h.steps), cudaMemcpyDeviceToHost,
                                 b->stream));
        SPH_CUDA(cudaMemcpyAsync(&h.err, b->d_err, sizeof(h.err), cudaMemcpyDeviceToHost,
                                 b->stream));
        SPH_CUDA(cudaStreamSynchronize(b->stream));
        const int done = (int)(h.steps - b->h_steps);
        b->h_steps = h.steps;
        if (h.err == 0u) break;
        // the failing step stopped where the error was raised; an RK2 step
        // may have stepped to its midpoint: back to the state it started from
        if (b->rec.scheme == 1) {
            for (int c = 0; c < 2 * b->rec.dim; ++c)
                SPH_CUDA(cudaMemcpyAsync(const_cast<double *>(state_ptr(b, c)), b->x0[c],
                                         sizeof(double) * b->view.n, cudaMemcpyDeviceToDevice,
                                         b->stream));
        }
        // a jump (or no margin to grow the regions by) is the caller's error
        // (the error word stays set for sph_batch_error_word)
        if ((h.err & ~SPH_EFLAG_BOX) != 0u || b->margin <= 0.0) break;
        stuck = done == 0 ? stuck + 1 : 0;
        if (stuck >= 3)
            return set_error(SPH_ERR_GRID, "batch: a particle keeps leaving its instance's region");
        rc = batch_regrid(b);
        if (rc) return rc;
        SPH_CUDA(cudaMemsetAsync(b->d_err, 0, sizeof(unsigned), b->stream));
        left -= done;
    }
    return SPH_OK;
}

__global__ void k_inst_pairs(const int *cnt, const int *sinst, int64_t n,
                             unsigned long long *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(out + sinst[i], (unsigned long long)cnt[i]);
}

int batch_pair_counts(sph_batch *b, unsigned long long *out) {
    if (!b->ready || b->steps_built == 0)
        return set_error(SPH_ERR_STATE, "batch: no evaluation yet");
    const size_t bytes = sizeof(unsigned long long) * b->ninst;
    if (!b->d_pairs) SPH_CUDA(cudaMalloc(&b->d_pairs, bytes));
    SPH_CUDA(cudaMemsetAsync(b->d_pairs, 0, bytes, b->stream));
    k_inst_pairs<<<grid_blocks(b->view.n, 256, 4), 256, 0, b->stream>>>(
        b->list.cnt, b->sinst, b->view.n, b->d_pairs);
    count_launch();
    SPH_LAUNCH_CHECK("k_inst_pairs");
    SPH_CUDA(cudaMemcpyAsync(out, b->d_pairs, bytes, cudaMemcpyDeviceToHost, b->stream));
    SPH_CUDA(cudaStreamSynchronize(b->stream));
    return SPH_OK;
}

void batch_free(sph_batch *b) {
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    ArraySnap &A = b->snap;
    cudaFree(A.key); cudaFree(A.perm); cudaFree(A.skey); cudaFree(A.scx); cudaFree(A.pm); cudaFree(A.velh);
    cudaFree(A.st); cudaFree(A.cstart); cudaFree(A.cursor); cudaFree(A.refcell);
    cudaFree(b->d_grids); cudaFree(b->d_inv_ref); cudaFree(b->inst_of); cudaFree(b->sinst);
    cudaFree(b->list.nbr); cudaFree(b->list.cnt); cudaFree(b->list.maxcnt);
    for (int c = 0; c < 6; ++c) {
        cudaFree(b->rate1[c]);
        cudaFree(b->rate2[c]);
        cudaFree(b->x0[c]);
    }
    cudaFree(b->d_err);
    cudaFree(b->d_pairs);
    cudaFree(b->d_off);
    cudaFree(b->d_ibox);
    cudaFree(b->d_steps);
}

}  // namespace sphgb
