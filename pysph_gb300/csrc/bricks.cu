// Brick-staged pair passes (sm_103a): the uniform-h summation density
// (+ Tait) and the PGrad + Monaghan AV (+ XSPH) rates of one simulation.
//
// Replaces, for the configurations it covers, the same reference routines
// as the list-streaming kernels of pairs.cu: SPHCalc.sph -> SPHFunction.eval
// -> eval_nbr over density_funcs.pyx:38-74 (SPHRho), eos_funcs.pyx:105-116
// (TaitEquation), pressure_funcs.pyx:40-91 (SPHPressureGradient),
// viscosity_funcs.pyx:41-124 (MonaghanArtificialVsicosity) and
// xsph_funcs.pyx:31-88 (XSPHCorrection), and the neighbour cache of
// base/nnps.pyx:566-620.
//
// One block owns one brick of bx * by * bz grid cells.  It copies the
// records of every source particle within the stencil half-width K of the
// brick -- the particles of the brick's rows of cells grown by K cells on
// every side -- once into shared memory, with positions relative to the
// brick's centre cell (FP32, |x| < ~12 cells, so |r_ab| keeps ~2e-7 of
// relative accuracy).  A destination's neighbour list then holds 16-bit
// indices into that staging, fixed between full builds (the sorted order and
// the cell table do not change), so a pair costs one list entry, shared-
// memory records and the pair arithmetic: no cell-offset decoding and no
// global gathers.  The entries of a destination are grouped by eight (one
// 16-byte load), groups of consecutive destinations adjacent, and the last
// group is padded with the index of a zero-mass record placed far away
// (index T, just past the staged records): the pair loop needs no bounds
// predicates.
//
// The neighbour relation is the reference's: strict r^2 < (radius_scale
// h)^2, decided in FP32 outside a +-1e-5 relative band around the threshold
// and by the FP64 test of base/nnps.pyx:337-353 inside it.  Neighbours are
// visited in the order of the list-streaming kernels (stencil rows in (dz,
// dy) order, ascending sorted slot within a row), and every destination's
// sums are Neumaier-compensated FP32 over plain batch partials.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <utility>
#include <vector>

#include "sph_internal.cuh"

namespace sphgb {

namespace {

// destination threads per block are chosen per build (the largest brick
// population rounded to warps); the kernels are compiled for at most this
constexpr int kBrickMaxThreads = 512;

struct BrickSrcDev {
    const float4 *pm, *velh, *st;
    const float *scx;
    const int *cstart, *perm;
    const double *x, *y, *z;
};

struct BrickDstDev {
    const float4 *pm, *velh, *st;
    const float *scx;
    const int *cstart, *perm;
    const int *bdst;       // exclusive prefix of the destinations per brick
    const int64_t *tag;
    const double *x, *y, *z, *h, *u, *v, *w, *p, *cs;
};

// shared-memory layout of a block (byte offsets into the dynamic array)
struct BrickSmem {
    int stage_cap;   // staged records (0: records are read from global memory)
    int off_v, off_s;             // rates: velocity / state records
    int off_rlo, off_roff, off_dlo, off_doff, off_scell;
};

// The neighbour radius of a uniform h, computed on the host with the
// operations of the per-destination test: radius2 = (h rs)^2 in FP64, its
// FP32 band [r2lo, r2hi] and the list radius r2list (0 without a skin).
struct BrickRadius {
    double radius2;
    float r2lo, r2hi, r2list;
};

struct BrickDensityArgs {
    Grid g;
    BrickGeom bk;
    BrickDstDev d;
    BrickSrcDev s;
    BrickSmem sm;
    BrickRadius rad;
    uint16_t *nbr;      // list: 8-entry group g of destination d of brick b is
                        // the uint4 (bdst[b] * cap / 8 + g * D_b + d)
    int *cnt;           // neighbour count per destination, brick order
    int *maxcnt;
    int cap;
    int build;          // 1: traverse the stencil and write the list
    int write_out;      // 0: list build only
    int dim, tait;
    float co, ro, gamma;
    double *rho_out, *p_out, *cs_out;
    float4 *st_out;
    const unsigned *gate;
};

struct BrickRatesArgs {
    Grid g;
    BrickGeom bk;
    BrickDstDev d;
    BrickSrcDev s;
    BrickSmem sm;
    BrickRadius rad;
    const uint16_t *nbr;
    const int *cnt;
    int cap;
    int dim;
    float alpha, beta, eta2, eps;
    int add_velocity, add_gravity, accumulate;
    // the sources' cs follows Tait with gamma = 7 from their rho (alpha cs /
    // 2 = tait_kc (rho / 2)^3): blocks whose sources share one mass then
    // read two records per pair instead of three
    int tait_state;
    float tait_kc;
    double gx, gy, gz;
    double *acc[3];
    double *pos[3];
    const unsigned *gate;
};

// The block's cells: brick [x0, x1) x [y0, y1) x [z0, z1), the staged
// region [xs0, xs1) x ... (the brick grown by the stencil half-widths,
// clipped to the grid) and the origin cell of the staged positions.
struct BlockGeo {
    int x0, x1, y0, y1, z0, z1;
    int xs0, xs1, ys0, ys1, zs0, zs1;
    int lx, ry, nr, dry, ndr;
    int cxc, cyc, czc;
};

__device__ __forceinline__ BlockGeo block_geo(const Grid &g, const BrickGeom &bk, int b) {
    BlockGeo G;
    const int ibx = b % bk.nbx;
    const int rest = b / bk.nbx;
    const int iby = rest % bk.nby;
    const int ibz = rest / bk.nby;
    G.x0 = ibx * bk.bx; G.x1 = min(g.nx, G.x0 + bk.bx);
    G.y0 = iby * bk.by; G.y1 = min(g.ny, G.y0 + bk.by);
    G.z0 = ibz * bk.bz; G.z1 = min(g.nz, G.z0 + bk.bz);
    G.xs0 = max(0, G.x0 - g.kx); G.xs1 = min(g.nx, G.x1 + g.kx);
    G.ys0 = max(0, G.y0 - g.ky); G.ys1 = min(g.ny, G.y1 + g.ky);
    G.zs0 = max(0, G.z0 - g.kz); G.zs1 = min(g.nz, G.z1 + g.kz);
    G.lx = G.xs1 - G.xs0;
    G.ry = G.ys1 - G.ys0;
    G.nr = G.ry * (G.zs1 - G.zs0);
    G.dry = G.y1 - G.y0;
    G.ndr = G.dry * (G.z1 - G.z0);
    G.cxc = G.x0 + bk.bx / 2;
    G.cyc = G.y0 + bk.by / 2;
    G.czc = G.z0 + bk.bz / 2;
    return G;
}

// In-place inclusive scan of a[1..n] by one warp (a[0] = 0 on return).
__device__ __forceinline__ void warp_scan_inplace(int *a, int n) {
    const int lane = threadIdx.x & 31;
    int carry = 0;
    for (int base = 1; base <= n; base += 32) {
        const int i = base + lane;
        int x = i <= n ? a[i] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (i <= n) a[i] = x + carry;
        carry += __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane == 0) a[0] = 0;
}

// Largest r in [0, n) with off[r] <= t (off[n] > t): the row holding index t.
__device__ __forceinline__ int row_of(const int *off, int n, int t) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= t) lo = mid; else hi = mid;
    }
    return lo;
}

// Position record (brick-relative x, y, z and the mass) of sorted slot j of
// row (cy, cz): the same FP32 operations for destinations and sources.
__device__ __forceinline__ float4 rel_pos(const float4 *pm, const float *scx, int j, int cy,
                                          int cz, const BlockGeo &G, float csf) {
    const float4 p = pm[j];
    return make_float4(fmaf(scx[j] - (float)G.cxc, csf, p.x),
                       fmaf((float)(cy - G.cyc), csf, p.y),
                       fmaf((float)(cz - G.czc), csf, p.z), p.w);
}

// Tables of a block: source rows (slot of the row's first staged cell and
// the staging offset of each row) and destination rows (the brick's rows of
// the destination array).  Returns the staged count and the destinations.
__device__ __forceinline__ void block_tables(const Grid &g, const BlockGeo &G, const int *scst,
                                             const int *dcst, int *rlo, int *roff, int *dlo,
                                             int *doff, int &T, int &D) {
    const int nt = blockDim.x;
    const int rowz = g.nx * g.ny;
    for (int r = threadIdx.x; r < G.nr; r += nt) {
        const int cy = G.ys0 + r % G.ry, cz = G.zs0 + r / G.ry;
        const int c = cz * rowz + cy * g.nx + G.xs0;
        const int lo = scst[c];
        rlo[r] = lo;
        roff[r + 1] = scst[c + G.lx] - lo;
    }
    for (int q = threadIdx.x; q < G.ndr; q += nt) {
        const int cy = G.y0 + q % G.dry, cz = G.z0 + q / G.dry;
        const int c = cz * rowz + cy * g.nx + G.x0;
        const int lo = dcst[c];
        dlo[q] = lo;
        doff[q + 1] = dcst[c + (G.x1 - G.x0)] - lo;
    }
    __syncthreads();
    const int wid = threadIdx.x >> 5;
    if (wid == 0) warp_scan_inplace(roff, G.nr);
    if (wid == (nt > 32 ? 1 : 0)) warp_scan_inplace(doff, G.ndr);
    __syncthreads();
    T = roff[G.nr];
    D = doff[G.ndr];
}

// Staging offset of the first particle of every cell of every source row
// (scell[r * (lx + 1) + i], i = 0 .. lx): the ranges a stencil traversal
// visits.
__device__ __forceinline__ void cell_table(const Grid &g, const BlockGeo &G, const int *scst,
                                           const int *rlo, const int *roff, int *scell) {
    const int w = G.lx + 1;
    const int rowz = g.nx * g.ny;
    for (int idx = threadIdx.x; idx < G.nr * w; idx += blockDim.x) {
        const int r = idx / w, i = idx - r * w;
        const int cy = G.ys0 + r % G.ry, cz = G.zs0 + r / G.ry;
        scell[idx] = roff[r] + (scst[cz * rowz + cy * g.nx + G.xs0 + i] - rlo[r]);
    }
}

// Sorted slot and row of staging index t (records read from global memory).
__device__ __forceinline__ int staged_slot(const BlockGeo &G, const int *rlo, const int *roff,
                                           int t, int &cy, int &cz) {
    const int r = row_of(roff, G.nr, t);
    cy = G.ys0 + r % G.ry;
    cz = G.zs0 + r / G.ry;
    return rlo[r] + (t - roff[r]);
}

// The dynamic shared memory of the brick kernels: the staged records from
// byte 0, then the block's tables.
extern __shared__ __align__(16) unsigned char brick_smem[];

// Table pointers and the state records' offset in the dynamic shared memory.
struct SmemPtrs {
    uint32_t voff, soff;
    int *rlo, *roff, *dlo, *doff, *scell;
};

__device__ __forceinline__ SmemPtrs smem_ptrs(unsigned char *base, const BrickSmem &sm) {
    SmemPtrs p;
    p.voff = (uint32_t)sm.off_v;
    p.soff = (uint32_t)sm.off_s;
    p.rlo = reinterpret_cast<int *>(base + sm.off_rlo);
    p.roff = reinterpret_cast<int *>(base + sm.off_roff);
    p.dlo = reinterpret_cast<int *>(base + sm.off_dlo);
    p.doff = reinterpret_cast<int *>(base + sm.off_doff);
    p.scell = reinterpret_cast<int *>(base + sm.off_scell);
    return p;
}

// The padding record (index T): far away, zero mass, at rest -- every pair
// term with it is exactly 0.
__device__ __forceinline__ float4 pad_pos() { return make_float4(1e15f, 1e15f, 1e15f, 0.f); }
__device__ __forceinline__ float4 pad_vel() { return make_float4(0.f, 0.f, 0.f, 0.f); }
// rates pass: the position record carries rho / 2, the state record (m,
// alpha cs / 2); the padding record has zero mass
__device__ __forceinline__ float4 pad_rpos() { return make_float4(1e15f, 1e15f, 1e15f, 0.5f); }
__device__ __forceinline__ float2 pad_rstate() { return make_float2(0.f, 0.f); }

// Source records: staged in shared memory, or (STAGED = false, a brick
// more populous than the shared memory holds) recomputed from the sorted
// arrays with the same operations.
template <bool STAGED, int PSH>
struct SrcRecords;

// Staged: the position record of source t at byte 16 t of the shared
// memory (x, y, z from the brick's centre cell, and m in the density pass,
// rho / 2 in the rates pass), in the rates pass the velocity record (u, v,
// w, p / rho^2) at voff + 16 t and the state record (m, alpha cs / 2) at
// soff + 8 t: 32-bit offsets into the shared array, so a record costs one
// address operation.  (Position and velocity interleaved in 32-byte
// records took 11 % longer: twice the bank conflicts of the random reads.)
// A rates pass whose block has one source mass and whose cs follows Tait
// (FAST) reads the first two only: the state record's 8-byte read was a
// fifth of the shared-memory wavefronts of a pair.
template <int PSH>
struct SrcRecords<true, PSH> {
    uint32_t voff, soff;
    __device__ __forceinline__ float4 pos(int t) const {
        return *reinterpret_cast<const float4 *>(brick_smem + ((uint32_t)t << 4));
    }
    // rates pass: position (w = rho / 2), velocity, mass, alpha cs / 2
    template <bool FAST>
    __device__ __forceinline__ void rates_rec(int t, float mb, float tkc, float4 &p, float4 &v,
                                              float &mj, float &hac) const {
        p = *reinterpret_cast<const float4 *>(brick_smem + ((uint32_t)t << 4));
        v = *reinterpret_cast<const float4 *>(brick_smem + voff + ((uint32_t)t << 4));
        if (FAST) {
            // cs = co (rho / ro)^3
            mj = mb;
            hac = tkc * (p.w * p.w) * p.w;
        } else {
            const float2 s = *reinterpret_cast<const float2 *>(brick_smem + soff + ((uint32_t)t << 3));
            mj = s.x;
            hac = s.y;
        }
    }
};

// recomputed from the sorted arrays with the staging's operations
template <int PSH>
struct SrcRecords<false, PSH> {
    const BrickSrcDev *src;
    BlockGeo G;
    const int *rlo, *roff;
    float csf;
    int T;
    float halpha;
    __device__ __forceinline__ float4 pos(int t) const {
        if (t >= T) return pad_pos();
        int cy, cz;
        const int j = staged_slot(G, rlo, roff, t, cy, cz);
        return rel_pos(src->pm, src->scx, j, cy, cz, G, csf);
    }
    template <bool FAST>
    __device__ __forceinline__ void rates_rec(int t, float, float, float4 &p, float4 &v, float &mj,
                                              float &hac) const {
        if (t >= T) {
            p = pad_rpos();
            v = pad_vel();
            mj = 0.f;
            hac = 0.f;
            return;
        }
        int cy, cz;
        const int j = staged_slot(G, rlo, roff, t, cy, cz);
        p = rel_pos(src->pm, src->scx, j, cy, cz, G, csf);
        const float4 vh = src->velh[j], st = src->st[j];
        mj = p.w;
        p.w = 0.5f * st.x;
        v = make_float4(vh.x, vh.y, vh.z, st.y);
        hac = halpha * st.z;
    }
};

template <bool STAGED, int PSH>
__device__ __forceinline__ SrcRecords<STAGED, PSH> make_records(const SmemPtrs &sp,
                                                                const BrickSrcDev &S,
                                                                const BlockGeo &G, float csf,
                                                                int T, float halpha) {
    if constexpr (STAGED)
        return SrcRecords<true, PSH>{sp.voff, sp.soff};
    else
        return SrcRecords<false, PSH>{&S, G, sp.rlo, sp.roff, csf, T, halpha};
}

// Copy the block's source records into shared memory (the layout of
// SrcRecords<true, .>).  Rates records: (x, y, z, rho / 2), (u, v, w,
// p / rho^2) and (m, alpha cs / 2), with the halves that the pair averages
// of the artificial viscosity add.  Returns whether every record this
// thread staged has mass mref.
template <bool RATES>
__device__ __forceinline__ bool stage(const BrickSrcDev &S, const BlockGeo &G, const int *rlo,
                                      const int *roff, int T, float csf, uint32_t voff,
                                      uint32_t soff, float halpha = 0.f, float mref = 0.f) {
    bool same = true;
    // unrolled so that several records' loads are in flight at once
#pragma unroll 4
    for (int t = threadIdx.x; t <= T; t += blockDim.x) {
        float4 *prec = reinterpret_cast<float4 *>(brick_smem + ((uint32_t)t << 4));
        float4 *vrec = reinterpret_cast<float4 *>(brick_smem + voff + ((uint32_t)t << 4));
        float2 *srec = reinterpret_cast<float2 *>(brick_smem + soff + ((uint32_t)t << 3));
        if (t == T) {
            // the padding record after the staged ones
            if (RATES) {
                *prec = pad_rpos();
                *vrec = pad_vel();
                *srec = pad_rstate();
            } else {
                *prec = pad_pos();
            }
            continue;
        }
        int cy, cz;
        const int j = staged_slot(G, rlo, roff, t, cy, cz);
        const float4 pr = rel_pos(S.pm, S.scx, j, cy, cz, G, csf);
        if (RATES) {
            const float4 vh = S.velh[j], st = S.st[j];
            *prec = make_float4(pr.x, pr.y, pr.z, 0.5f * st.x);
            *vrec = make_float4(vh.x, vh.y, vh.z, st.y);
            *srec = make_float2(pr.w, halpha * st.z);
            same = same && pr.w == mref;
        } else {
            *prec = pr;
        }
    }
    return same;
}

// The 16-bit entry i (0..7) of a group.
__device__ __forceinline__ int group_entry(const uint4 &q, int i) {
    const unsigned w = i < 2 ? q.x : (i < 4 ? q.y : (i < 6 ? q.z : q.w));
    return (int)((i & 1) ? (w >> 16) : (w & 0xffffu));
}

// One destination of the block.
struct BrickDest {
    int s;          // sorted slot
    int orig;       // original index
    int cx, cy, cz; // build cell
    float xi_x, xi_y, xi_z;     // cell-local offsets (stencil pruning)
    float4 P;       // brick-relative position, mass
    float r2lo, r2hi, r2list;
    double radius2;
};

__device__ __forceinline__ bool brick_dest(const Grid &g, const BrickDstDev &D, const BlockGeo &G,
                                           const BrickRadius &rad, const int *dlo,
                                           const int *doff, int d, BrickDest &q) {
    const int r = row_of(doff, G.ndr, d);
    q.s = dlo[r] + (d - doff[r]);
    q.cy = G.y0 + r % G.dry;
    q.cz = G.z0 + r / G.dry;
    q.orig = D.perm[q.s];
    const float4 p = D.pm[q.s];
    q.xi_x = p.x; q.xi_y = p.y; q.xi_z = p.z;
    q.cx = (int)D.scx[q.s];
    q.P = rel_pos(D.pm, D.scx, q.s, q.cy, q.cz, G, g.cs_f);
    q.radius2 = rad.radius2;
    q.r2lo = rad.r2lo;
    q.r2hi = rad.r2hi;
    q.r2list = rad.r2list;
    return D.tag == nullptr || D.tag[q.orig] == SPH_TAG_LOCAL_REAL;
}

// Visit the listed sources of destination q in the staged records, in the
// order of the list-streaming kernels: stencil rows in (dz, dy) order, each
// clipped to the chord of the search sphere, ascending slot within a row.
// fn(t, rx, ry, rz, hit): staging index, r = x_dest - x_src, neighbour or
// (with a list skin) only within the list radius.  The ranges come from the
// block's cell table (scell) or, without one, from the grid's cell table.
template <int K, bool STAGED, int PSH, class Fn>
__device__ __forceinline__ void brick_traverse(const Grid &g, const BlockGeo &G, const BrickSrcDev &S,
                                               const BrickDstDev &D, const SrcRecords<STAGED, PSH> &R,
                                               const int *rlo, const int *roff, const int *scell,
                                               const BrickDest &q, Fn &&fn) {
    const float csf = g.cs_f;
    const float inv_cs = 1.f / csf;
    const float R2 = fmaxf(q.r2hi, q.r2list) * 1.0002f;
    const int w = G.lx + 1;
#pragma unroll 1
    for (int dz = -g.kz; dz <= g.kz; ++dz) {
        const int czz = q.cz + dz;
        if (czz < G.zs0 || czz >= G.zs1) continue;
        const float ez = fmaxf(0.f, dz > 0 ? (float)dz * csf - q.xi_z
                                           : (dz < 0 ? q.xi_z - (float)(dz + 1) * csf : 0.f));
        const float ez2 = ez * ez;
        if (ez2 > R2) continue;
#pragma unroll 1
        for (int dy = -g.ky; dy <= g.ky; ++dy) {
            const int cyy = q.cy + dy;
            if (cyy < G.ys0 || cyy >= G.ys1) continue;
            const float ey = fmaxf(0.f, dy > 0 ? (float)dy * csf - q.xi_y
                                               : (dy < 0 ? q.xi_y - (float)(dy + 1) * csf : 0.f));
            const float rem = R2 - fmaf(ey, ey, ez2);
            if (rem < 0.f) continue;
            const float half = fmaf(rem * rsqrtf(fmaxf(rem, 1e-30f)), 1.0001f, 1e-5f * csf);
            const int tlo = max(-K, __float2int_rd((q.xi_x - half) * inv_cs));
            const int thi = min(K, __float2int_rd((q.xi_x + half) * inv_cs));
            const int clo = max(q.cx + tlo, G.xs0);
            const int chi = min(q.cx + thi, G.xs1 - 1);
            if (clo > chi) continue;
            const int rr = (cyy - G.ys0) + G.ry * (czz - G.zs0);
            int ta, tb;
            if (scell != nullptr) {
                ta = scell[rr * w + (clo - G.xs0)];
                tb = scell[rr * w + (chi + 1 - G.xs0)];
            } else {
                const int c = (czz * g.ny + cyy) * g.nx;
                ta = roff[rr] + (__ldg(S.cstart + c + clo) - rlo[rr]);
                tb = roff[rr] + (__ldg(S.cstart + c + chi + 1) - rlo[rr]);
            }
            for (int t = ta; t < tb; ++t) {
                const float4 pj = R.pos(t);
                const float rx = q.P.x - pj.x, ry = q.P.y - pj.y, rz = q.P.z - pj.z;
                const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                bool hit = r2 < q.r2lo;
                if (!hit && r2 <= q.r2hi) {
                    const int oj = S.perm[rlo[rr] + (t - roff[rr])];
                    hit = exact_within(ld0(S.x, oj), ld0(S.y, oj), ld0(S.z, oj), ld0(D.x, q.orig),
                                       ld0(D.y, q.orig), ld0(D.z, q.orig), q.radius2);
                }
                if (hit || r2 < q.r2list) fn(t, rx, ry, rz, hit);
            }
        }
    }
}

// Reciprocal square root and reciprocal, flushing subnormal inputs to zero
// (the pair terms' inputs are bounded away from the subnormal range: r^2 is
// clamped to 1e-30, the density sums are near the rest density).
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ bool gate_off(const unsigned *gate) {
    return gate != nullptr && __ldg(gate) != 0u;
}

// ---------------------------------------------------------------------------
// summation density (density_funcs.pyx:38-74) + Tait (eos_funcs.pyx:105-116)
// ---------------------------------------------------------------------------
// fac W(q) of the cubic spline (base/kernels.pyx:351-374), the normalisation
// (and any constant factor) folded into the coefficients: fac (1 - 1.5 q^2
// + 0.75 q^3) for q <= 1, fac / 4 (2 - q)^3 for 1 < q <= 2, else 0.
struct WCoef {
    float i0, i1, i2, o;
};

__device__ __forceinline__ WCoef w_coef(float fac, float scale) {
    const float f = fac * scale;
    return WCoef{f, -1.5f * f, 0.75f * f, 0.25f * f};
}

__device__ __forceinline__ float w_of(float q, const WCoef &c) {
    const float inner = fmaf(q * q, fmaf(c.i2, q, c.i1), c.i0);
    const float t = 2.f - q;
    const float outer = c.o * (t * t) * t;
    return q > 2.f ? 0.f : (q > 1.f ? outer : inner);
}

__device__ __forceinline__ float density_term(const float4 &pi, const float4 &pj, float ih,
                                              const WCoef &wc) {
    const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
    const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
    const float r = r2 * rsqrt_ftz(fmaxf(r2, 1e-30f));
    return w_of(r * ih, wc) * pj.w;
}

// Density of one destination (the compensated sum hi + lo) and, with
// Tait, its p and cs; the sorted state record when the pass writes the
// destination's own properties.
__device__ __forceinline__ void density_store(const BrickDensityArgs &A, int s, int orig, bool real,
                                              float hi, float lo) {
    const double r64 = (double)hi + (double)lo;
    if (A.rho_out) A.rho_out[orig] = r64;
    const float rf = hi + lo;
    float pf = 0.f, cf = 0.f;
    if (A.tait) {
        if (real) {
            // p = B((rho/ro)^gamma - 1), cs = co (rho/ro)^((gamma-1)/2), through
            // log1p/expm1 of the density excess (relative accuracy of p as
            // rho -> ro); hi - ro is exact for hi within a factor 2 of ro
            const float Bt = A.co * A.co * A.ro / A.gamma;
            const float lr = log1pf(((hi - A.ro) + lo) * (1.f / A.ro));
            pf = Bt * expm1f(A.gamma * lr);
            cf = A.co * expf(0.5f * (A.gamma - 1.f) * lr);
        }
        A.p_out[orig] = (double)pf;
        A.cs_out[orig] = (double)cf;
    }
    if (A.st_out) {
        const float mi = A.d.pm[s].w;
        if (A.tait) {
            A.st_out[s] = make_float4(rf, pf / (rf * rf), cf, mi);
        } else {
            const float pold = (float)ld0(A.d.p, orig);
            A.st_out[s] = make_float4(rf, pold / (rf * rf), (float)ld0(A.d.cs, orig), mi);
        }
    }
}

// What a destination's sums start from: its slot and records, its count
// and the first two groups of its list.  The first destination of every
// thread requests these before the block stages its sources, so their
// latency overlaps the staging.
struct DestPre {
    int s, orig;    // sorted slot, original index
    bool real;
    float4 P;       // brick-relative position, mass
    int c;
    uint4 b0, b1;
};

__device__ __forceinline__ void dest_prefetch(const BrickDstDev &Dd, const Grid &g,
                                              const BlockGeo &G, const BrickRadius &rad,
                                              const SmemPtrs &sp, const int *cnt,
                                              const uint4 *lgrp, int cap, int D, int dbase,
                                              int d, DestPre &p) {
    BrickDest q;
    p.real = brick_dest(g, Dd, G, rad, sp.dlo, sp.doff, d, q);
    p.s = q.s;
    p.orig = q.orig;
    p.P = q.P;
    p.c = cnt[dbase + d];
    // every destination owns cap / 8 groups: the first two are read whatever
    // the count (used only as far as it reaches)
    const uint4 *lst = lgrp + d;
    p.b0 = lst[0];
    p.b1 = cap >= 16 ? lst[D] : make_uint4(0, 0, 0, 0);
}

// The density sum of one destination over its list: groups of 8 entries,
// each requested two groups ahead into one of three rotating buffers.
template <bool STAGED, int PSH>
__device__ __forceinline__ void density_group(CSum &rho, const SrcRecords<STAGED, PSH> &R,
                                              const uint4 &grp, const float4 &Pi, float ih,
                                              const WCoef &wc) {
    float part = 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float4 pj[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) pj[i] = R.pos(group_entry(grp, 4 * h + i));
#pragma unroll
        for (int i = 0; i < 4; ++i) part += density_term(Pi, pj[i], ih, wc);
    }
    rho.add(part);
}

template <bool STAGED, int PSH>
__device__ __forceinline__ void density_stream(CSum &rho, const SrcRecords<STAGED, PSH> &R,
                                               const uint4 *lst, int D, int ng, const float4 &Pi,
                                               float ih, const WCoef &wc, uint4 b0, uint4 b1) {
    const uint4 zero = make_uint4(0, 0, 0, 0);
    const size_t step = (size_t)D;
    uint4 b2;
    for (int gi = 0;;) {
        if (gi >= ng) break;
        b2 = gi + 2 < ng ? lst[(gi + 2) * step] : zero;
        density_group<STAGED>(rho, R, b0, Pi, ih, wc);
        if (++gi >= ng) break;
        b0 = gi + 2 < ng ? lst[(gi + 2) * step] : zero;
        density_group<STAGED>(rho, R, b1, Pi, ih, wc);
        if (++gi >= ng) break;
        b1 = gi + 2 < ng ? lst[(gi + 2) * step] : zero;
        density_group<STAGED>(rho, R, b2, Pi, ih, wc);
        ++gi;
    }
}

template <int K, bool BUILD, bool STAGED>
__global__ void __maxnreg__(64) k_bdensity(const __grid_constant__ BrickDensityArgs A) {
    unsigned char *smem = brick_smem;
    if (gate_off(A.gate)) return;
    const int b = blockIdx.x;
    const int nd = A.d.bdst[b + 1] - A.d.bdst[b];
    if (nd == 0) return;
    const Grid &g = A.g;
    const BlockGeo G = block_geo(g, A.bk, b);
    SmemPtrs sp = smem_ptrs(smem, A.sm);
    int T, D;
    block_tables(g, G, A.s.cstart, A.d.cstart, sp.rlo, sp.roff, sp.dlo, sp.doff, T, D);
    const int dbase = A.d.bdst[b];
    const int cap = A.cap;            // a multiple of 8
    const int ng_cap = cap >> 3;
    // the stencil cell table of a list build (a destination whose neighbours
    // outgrew the list reads the grid's table instead)
    int *scell = BUILD ? sp.scell : nullptr;
    const uint4 *lgrp = reinterpret_cast<const uint4 *>(A.nbr) + (size_t)dbase * ng_cap;
    // the first destination of this thread, requested before the staging
    DestPre pre;
    if (!BUILD && (int)threadIdx.x < D)
        dest_prefetch(A.d, g, G, A.rad, sp, A.cnt, lgrp, cap, D, dbase, threadIdx.x, pre);
    if (BUILD) cell_table(g, G, A.s.cstart, sp.rlo, sp.roff, sp.scell);
    if (STAGED) stage<false>(A.s, G, sp.rlo, sp.roff, T, g.cs_f, sp.voff, sp.soff);
    __syncthreads();
    const SrcRecords<STAGED, 4> R = make_records<STAGED, 4>(sp, A.s, G, g.cs_f, T, 0.f);
    const float ih = __fdividef(1.f, g.h_uniform);
    const float fac = cubic_fac(A.dim, ih);
    const WCoef wc = w_coef(fac, 1.f);
    // destination d from its record p (for a list build, the traversal fills it)
    auto one = [&](int d, DestPre &p) {
        BrickDest q;
        if (BUILD) {
            p.real = brick_dest(g, A.d, G, A.rad, sp.dlo, sp.doff, d, q);
            p.s = q.s;
            p.orig = q.orig;
        }
        const bool real = p.real;
        CSum rho;
        int c = 0;
        if (real) {
            if (BUILD) {
                // entries collected eight at a time in a 128-bit shift
                // register (the newest enters at the top) and written as
                // one 16-byte store per group
                uint4 *out = reinterpret_cast<uint4 *>(A.nbr) + (size_t)dbase * ng_cap + d;
                uint4 grp = make_uint4(0, 0, 0, 0);
                auto push = [&](unsigned t) {
                    grp.x = __funnelshift_r(grp.x, grp.y, 16);
                    grp.y = __funnelshift_r(grp.y, grp.z, 16);
                    grp.z = __funnelshift_r(grp.z, grp.w, 16);
                    grp.w = (grp.w >> 16) | (t << 16);
                };
                // neighbours summed in plain FP32 batches of 8 hits, each
                // batch folded into the compensated sum
                float part = 0.f;
                int nb = 0;
                brick_traverse<K, STAGED>(g, G, A.s, A.d, R, sp.rlo, sp.roff, scell, q,
                    [&](int t, float rx, float ry, float rz, bool hit) {
                        if (c < cap) {
                            push((unsigned)t);
                            if ((c & 7) == 7) out[(size_t)(c >> 3) * D] = grp;
                        }
                        ++c;
                        if (!hit) return;
                        const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                        const float r = r2 * rsqrt_ftz(fmaxf(r2, 1e-30f));
                        part += w_of(r * ih, wc) * R.pos(t).w;
                        if (++nb == 8) {
                            rho.add(part);
                            part = 0.f;
                            nb = 0;
                        }
                    });
                rho.add(part);
                // pad the last group with the zero record
                if (c < cap && (c & 7)) {
                    for (int k = c; k & 7; ++k) push((unsigned)T);
                    out[(size_t)(c >> 3) * D] = grp;
                }
            } else {
                c = p.c;
                density_stream<STAGED>(rho, R, lgrp + d, D, (min(c, cap) + 7) >> 3, p.P, ih, wc,
                                       p.b0, p.b1);
            }
        }
        if (BUILD) {
            A.cnt[dbase + d] = c;
            const unsigned act = __activemask();
            const int wmax = __reduce_max_sync(act, c);
            if ((threadIdx.x & 31) == (__ffs(act) - 1)) atomicMax(A.maxcnt, wmax);
        }
        if (A.write_out)
            density_store(A, p.s, p.orig, real, real ? rho.hi : 0.f, real ? rho.lo : 0.f);
    };
    for (int d = threadIdx.x; d < D; d += blockDim.x) {
        if (!BUILD && d != (int)threadIdx.x)
            dest_prefetch(A.d, g, G, A.rad, sp, A.cnt, lgrp, cap, D, dbase, d, pre);
        one(d, pre);
    }
    if constexpr (BUILD) return;
    if (!A.write_out || A.rho_out == nullptr) return;
    // destinations with more neighbours than their list holds: the rest
    // come from a traversal that skips the listed ones (in the order of
    // the list build), added to the stored partial density
    for (int d = threadIdx.x; d < D; d += blockDim.x) {
        if (A.cnt[dbase + d] <= cap) continue;
        BrickDest q;
        if (!brick_dest(g, A.d, G, A.rad, sp.dlo, sp.doff, d, q)) continue;
        CSum rest;
        int skip = cap;
        brick_traverse<K, STAGED>(g, G, A.s, A.d, R, sp.rlo, sp.roff, nullptr, q,
            [&](int t, float rx, float ry, float rz, bool hit) {
                if (skip > 0) { --skip; return; }
                if (!hit) return;
                const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                const float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
                rest.add(cubic_w(r * ih) * fac * R.pos(t).w);
            });
        // the stored partial density (hi + lo of the listed part, in FP64)
        // plus the rest, as a compensated FP32 pair
        CSum tot = rest;
        const double part = A.rho_out[q.orig];
        const float phi = (float)part;
        tot.merge(phi, (float)(part - (double)phi));
        density_store(A, q.s, q.orig, true, tot.hi, tot.lo);
    }
}

// ---------------------------------------------------------------------------
// rates: PGrad (pressure_funcs.pyx:40-91) + Monaghan AV (viscosity_funcs.pyx:
// 41-124) [+ XSPH (xsph_funcs.pyx:31-88)], uniform h, one source, with
// gravity (external_force.pyx:39-45) and position stepping
// (position_funcs.pyx:32-60) folded into the store
// ---------------------------------------------------------------------------
struct RatesConst {
    float h, ih, beta, eta2h2;
    float gin0, gin1, gout;     // fac dW/dr / r: gin1 q + gin0 (q < 1), gout (2-q)^2 / r (q < 2)
    WCoef wx;                   // eps fac W(q) (XSPH)
    float mb, tkc;              // two-record blocks: the sources' mass, alpha cs / 2 per (rho / 2)^3
};

__device__ __forceinline__ RatesConst rates_const(float h, float fac, float beta, float eta2,
                                                  float eps) {
    RatesConst k;
    k.h = h;
    k.ih = __fdividef(1.f, h);
    k.beta = beta;
    k.eta2h2 = eta2 * h * h;
    // fac 3 (0.75 q - 1) / h^2 and -0.75 fac (2 - q)^2 / (h r) (base/kernels.pyx:376-413)
    k.gin1 = 2.25f * fac * k.ih * k.ih;
    k.gin0 = -3.f * fac * k.ih * k.ih;
    k.gout = -0.75f * fac * k.ih;
    k.wx = w_coef(fac, eps);
    k.mb = 0.f;
    k.tkc = 0.f;
    return k;
}

// destination state and the sums: plain FP32 partials of a batch, merged
// into the Neumaier-compensated totals by flush()
struct RatesAcc {
    float4 vi;
    float hrhoi, pri, haci;     // rho_i / 2, p_i / rho_i^2, alpha cs_i / 2
    float pax, pay, paz, pxx, pxy, pxz;
    CSum ax, ay, az, xx, xy, xz;
};

// One pair: pressure gradient -m_j (p_i/rho_i^2 + p_j/rho_j^2) grad W
// (pressure_funcs.pyx:67-91), Monaghan viscosity -m_j Pi_ab grad W with
// mu = h v_ab.r_ab / (r^2 + eta^2 h^2) for approaching pairs
// (viscosity_funcs.pyx:72-124; min(v.r, 0) gives mu = 0 otherwise, and
// with eta = 0, as the reference's class always has, 1/r^2 comes from the
// rsqrt already taken), and XSPH eps m_j W (v_j - v_i) / rho_ab
// (xsph_funcs.pyx:44-88), sharing 1 / rho_ab.
// Source record: pj = (position, rho_j / 2), vj = (velocity, p_j / rho_j^2),
// mj, hacj = alpha cs_j / 2.
template <bool XSPH, bool ETA0>
__device__ __forceinline__ void rates_pair(RatesAcc &a, const RatesConst &k, float rx, float ry,
                                           float rz, const float4 &pj, const float4 &vj,
                                           float mj, float hacj) {
    const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
    const float rinv = rsqrt_ftz(fmaxf(r2, 1e-30f));
    const float q = r2 * rinv * k.ih;
    const float dot = (a.vi.x - vj.x) * rx + (a.vi.y - vj.y) * ry + (a.vi.z - vj.z) * rz;
    const float hdot = k.h * fminf(dot, 0.f);
    const float mu = ETA0 ? hdot * rinv * rinv : __fdividef(hdot, r2 + k.eta2h2);
    const float inv_rhoab = rcp_ftz(a.hrhoi + pj.w);
    const float piab = mu * fmaf(k.beta, mu, -(a.haci + hacj)) * inv_rhoab;
    const float t = -mj * ((a.pri + vj.w) + piab);
    // (2 - q) clamped at 0: the outer branch is 0 beyond q = 2
    const float tq = fmaxf(2.f - q, 0.f);
    const float g = q >= 1.f ? k.gout * (tq * tq) * rinv : fmaf(k.gin1, q, k.gin0);
    const float gf = g * t;
    a.pax = fmaf(gf, rx, a.pax);
    a.pay = fmaf(gf, ry, a.pay);
    a.paz = fmaf(gf, rz, a.paz);
    if (XSPH) {
        const float temp = mj * w_of(q, k.wx) * inv_rhoab;
        a.pxx = fmaf(temp, vj.x - a.vi.x, a.pxx);
        a.pxy = fmaf(temp, vj.y - a.vi.y, a.pxy);
        a.pxz = fmaf(temp, vj.z - a.vi.z, a.pxz);
    }
}

template <bool XSPH>
__device__ __forceinline__ void rates_flush(RatesAcc &a) {
    a.ax.add(a.pax); a.ay.add(a.pay); a.az.add(a.paz);
    a.pax = a.pay = a.paz = 0.f;
    if (XSPH) {
        a.xx.add(a.pxx); a.xy.add(a.pxy); a.xz.add(a.pxz);
        a.pxx = a.pxy = a.pxz = 0.f;
    }
}

// The pairs of one group of 8 list entries, records two at a time, then
// the batch's partial sums folded into the compensated ones.
template <bool XSPH, bool ETA0, bool FAST, bool STAGED, int PSH>
__device__ __forceinline__ void rates_group(RatesAcc &acc, const RatesConst &kc,
                                            const SrcRecords<STAGED, PSH> &R, const uint4 &grp,
                                            const float4 &Pi) {
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        float4 pj[2], vj[2];
        float mj[2], hac[2];
#pragma unroll
        for (int i = 0; i < 2; ++i)
            R.template rates_rec<FAST>(group_entry(grp, 2 * h + i), kc.mb, kc.tkc, pj[i], vj[i],
                                       mj[i], hac[i]);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            rates_pair<XSPH, ETA0>(acc, kc, Pi.x - pj[i].x, Pi.y - pj[i].y, Pi.z - pj[i].z,
                                   pj[i], vj[i], mj[i], hac[i]);
    }
    rates_flush<XSPH>(acc);
}

// The sums of one destination: its list streamed in groups of 8 entries,
// each group requested two groups ahead into one of three rotating
// buffers (the loop body is unrolled over the three, so no buffer is
// copied).
template <bool XSPH, bool ETA0, bool FAST, bool STAGED, int PSH>
__device__ __forceinline__ void rates_stream(RatesAcc &acc, const RatesConst &kc,
                                             const SrcRecords<STAGED, PSH> &R, const uint4 *lst, int D,
                                             int ng, const float4 &Pi, uint4 b0, uint4 b1) {
    const uint4 zero = make_uint4(0, 0, 0, 0);
    uint4 b2;
    const size_t step = (size_t)D;
    for (int gi = 0;;) {
        if (gi >= ng) break;
        b2 = gi + 2 < ng ? lst[(gi + 2) * step] : zero;
        rates_group<XSPH, ETA0, FAST, STAGED>(acc, kc, R, b0, Pi);
        if (++gi >= ng) break;
        b0 = gi + 2 < ng ? lst[(gi + 2) * step] : zero;
        rates_group<XSPH, ETA0, FAST, STAGED>(acc, kc, R, b1, Pi);
        if (++gi >= ng) break;
        b1 = gi + 2 < ng ? lst[(gi + 2) * step] : zero;
        rates_group<XSPH, ETA0, FAST, STAGED>(acc, kc, R, b2, Pi);
        ++gi;
    }
}

// Neighbours of destination q past its list's capacity: a traversal that
// skips the listed ones (in the order of the list build).
template <int K, bool XSPH, bool ETA0, bool STAGED, int PSH>
__device__ __forceinline__ void rates_rest(RatesAcc &acc, const RatesConst &kc, const Grid &g,
                                           const BlockGeo &G, const BrickSrcDev &S,
                                           const BrickDstDev &D, const SrcRecords<STAGED, PSH> &R,
                                           const int *rlo, const int *roff, const BrickDest &q,
                                           int cap) {
    int skip = cap;
    brick_traverse<K, STAGED>(g, G, S, D, R, rlo, roff, nullptr, q,
        [&](int t, float rx, float ry, float rz, bool hit) {
            if (skip > 0) { --skip; return; }
            if (!hit) return;
            float4 pj, vj;
            float mj, hac;
            R.template rates_rec<false>(t, 0.f, 0.f, pj, vj, mj, hac);
            rates_pair<XSPH, ETA0>(acc, kc, rx, ry, rz, pj, vj, mj, hac);
            rates_flush<XSPH>(acc);
        });
}

__device__ __forceinline__ void rates_acc_init(RatesAcc &acc, const float4 &vi, const float4 &st,
                                               float halpha) {
    acc.pax = acc.pay = acc.paz = acc.pxx = acc.pxy = acc.pxz = 0.f;
    acc.vi = vi;
    acc.hrhoi = 0.5f * st.x;
    acc.pri = st.y;
    acc.haci = halpha * st.z;
}

// The sums of destination d (listed part) and their store.
template <bool XSPH, bool ETA0, bool FAST, bool STAGED, int PSH>
__device__ __forceinline__ void rates_dest(const BrickRatesArgs &A, const SrcRecords<STAGED, PSH> &R,
                                           const RatesConst &kc, const uint4 *lgrp, int D, int d,
                                           const DestPre &pre) {
    const int cap = A.cap;
    const bool real = pre.real;
    RatesAcc acc;
    rates_acc_init(acc, A.d.velh[pre.s], A.d.st[pre.s], 0.5f * A.alpha);
    if (real)
        rates_stream<XSPH, ETA0, FAST, STAGED>(acc, kc, R, lgrp + d, D, (min(pre.c, cap) + 7) >> 3,
                                         pre.P, pre.b0, pre.b1);
    const int orig = pre.orig;
    double a3[3] = {0.0, 0.0, 0.0}, p3[3] = {0.0, 0.0, 0.0};
    if (real) {
        // the compensated sums rounded once to FP32 (far below the pair
        // terms' own FP32 error), one conversion each
        a3[0] = (double)acc.ax.fvalue(); a3[1] = (double)acc.ay.fvalue();
        a3[2] = (double)acc.az.fvalue();
        if (XSPH) {
            p3[0] = (double)acc.xx.fvalue(); p3[1] = (double)acc.xy.fvalue();
            p3[2] = (double)acc.xz.fvalue();
        }
        if (A.add_gravity) { a3[0] += A.gx; a3[1] += A.gy; a3[2] += A.gz; }
        if (A.add_velocity) {
            // exact FP64 velocity of the destination (position_funcs.pyx:47-50)
            p3[0] += ld0(A.d.u, orig);
            p3[1] += ld0(A.d.v, orig);
            p3[2] += ld0(A.d.w, orig);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (A.acc[k]) A.acc[k][orig] = (A.accumulate ? A.acc[k][orig] : 0.0) + a3[k];
        if (A.pos[k]) A.pos[k][orig] = (A.accumulate ? A.pos[k][orig] : 0.0) + p3[k];
    }
}

template <int K, bool XSPH, bool ETA0, bool FAST, bool STAGED, int PSH>
__device__ __forceinline__ void rates_block(const BrickRatesArgs &A, const Grid &g,
                                            const BlockGeo &G, const SmemPtrs &sp,
                                            const SrcRecords<STAGED, PSH> &R, const RatesConst &kc,
                                            int D, int dbase, const DestPre &first) {
    const int cap = A.cap;
    const float halpha = 0.5f * A.alpha;
    const uint4 *lgrp = reinterpret_cast<const uint4 *>(A.nbr) + (size_t)dbase * (cap >> 3);
    // the first destination of the thread from its prefetched record, the
    // others (bricks with more destinations than threads) as they come
    if ((int)threadIdx.x < D)
        rates_dest<XSPH, ETA0, FAST, STAGED>(A, R, kc, lgrp, D, threadIdx.x, first);
    for (int d = threadIdx.x + blockDim.x; d < D; d += blockDim.x) {
        DestPre pre;
        dest_prefetch(A.d, g, G, A.rad, sp, A.cnt, lgrp, cap, D, dbase, d, pre);
        rates_dest<XSPH, ETA0, FAST, STAGED>(A, R, kc, lgrp, D, d, pre);
    }
    // destinations with more neighbours than their list holds: the rest
    // added to the stored sums
    for (int d = threadIdx.x; d < D; d += blockDim.x) {
        if (A.cnt[dbase + d] <= cap) continue;
        BrickDest q;
        if (!brick_dest(g, A.d, G, A.rad, sp.dlo, sp.doff, d, q)) continue;
        RatesAcc acc;
        rates_acc_init(acc, A.d.velh[q.s], A.d.st[q.s], halpha);
        rates_rest<K, XSPH, ETA0, STAGED>(acc, kc, g, G, A.s, A.d, R, sp.rlo, sp.roff, q, cap);
        const double a3[3] = {(double)acc.ax.fvalue(), (double)acc.ay.fvalue(),
                              (double)acc.az.fvalue()};
        const double p3[3] = {(double)acc.xx.fvalue(), (double)acc.xy.fvalue(),
                              (double)acc.xz.fvalue()};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (A.acc[k]) A.acc[k][q.orig] += a3[k];
            if (A.pos[k]) A.pos[k][q.orig] += p3[k];
        }
    }
}

template <int K, bool XSPH, bool STAGED>
__global__ void __maxnreg__(XSPH ? 80 : 64) k_brates(const __grid_constant__ BrickRatesArgs A) {
    unsigned char *smem = brick_smem;
    if (gate_off(A.gate)) return;
    const int b = blockIdx.x;
    const int nd = A.d.bdst[b + 1] - A.d.bdst[b];
    if (nd == 0) return;
    const Grid &g = A.g;
    const BlockGeo G = block_geo(g, A.bk, b);
    SmemPtrs sp = smem_ptrs(smem, A.sm);
    int T, D;
    block_tables(g, G, A.s.cstart, A.d.cstart, sp.rlo, sp.roff, sp.dlo, sp.doff, T, D);
    const int dbase = A.d.bdst[b];
    DestPre pre;
    if ((int)threadIdx.x < D) {
        const uint4 *lgrp = reinterpret_cast<const uint4 *>(A.nbr) + (size_t)dbase * (A.cap >> 3);
        dest_prefetch(A.d, g, G, A.rad, sp, A.cnt, lgrp, A.cap, D, dbase, threadIdx.x, pre);
    }
    const float halpha = 0.5f * A.alpha;
    // two-record blocks: staged sources of one mass (that of the first) whose
    // cs follows Tait
    const bool try_fast = STAGED && A.tait_state != 0 && A.eta2 == 0.f && T > 0;
    float mref = 0.f;
    if (try_fast) {
        int cy, cz;
        mref = A.s.pm[staged_slot(G, sp.rlo, sp.roff, 0, cy, cz)].w;
    }
    bool same = true;
    if (STAGED) same = stage<true>(A.s, G, sp.rlo, sp.roff, T, g.cs_f, sp.voff, sp.soff, halpha, mref);
    const bool fast = __syncthreads_and(try_fast && same) != 0;
    const SrcRecords<STAGED, 5> R = make_records<STAGED, 5>(sp, A.s, G, g.cs_f, T, halpha);
    const float ih = __fdividef(1.f, g.h_uniform);
    RatesConst kc = rates_const(g.h_uniform, cubic_fac(A.dim, ih), A.beta, A.eta2, A.eps);
    if (A.eta2 == 0.f) {
        if constexpr (STAGED) {
            if (fast) {
                kc.mb = mref;
                kc.tkc = A.tait_kc;
                rates_block<K, XSPH, true, true, STAGED>(A, g, G, sp, R, kc, D, dbase, pre);
                return;
            }
        }
        rates_block<K, XSPH, true, false, STAGED>(A, g, G, sp, R, kc, D, dbase, pre);
    } else {
        rates_block<K, XSPH, false, false, STAGED>(A, g, G, sp, R, kc, D, dbase, pre);
    }
}

// ---------------------------------------------------------------------------
// per-brick tables of one array: destinations per brick (then scanned into
// bdst) and the largest count of source particles a brick stages
// ---------------------------------------------------------------------------
__global__ void k_brick_tables(Grid g, BrickGeom bk, const int *cstart, int *dcount,
                               unsigned *stats) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    unsigned tmax = 0, dmax = 0;
    if (b < bk.nbricks) {
        const BlockGeo G = block_geo(g, bk, (int)b);
        const int rowz = g.nx * g.ny;
        int D = 0;
        for (int cz = G.z0; cz < G.z1; ++cz)
            for (int cy = G.y0; cy < G.y1; ++cy) {
                const int c = cz * rowz + cy * g.nx;
                D += cstart[c + G.x1] - cstart[c + G.x0];
            }
        // every brick: as a source this array is staged by the bricks that
        // hold destinations of any array
        int T = 0;
        for (int cz = G.zs0; cz < G.zs1; ++cz)
            for (int cy = G.ys0; cy < G.ys1; ++cy) {
                const int c = cz * rowz + cy * g.nx;
                T += cstart[c + G.xs1] - cstart[c + G.xs0];
            }
        dcount[b] = D;
        tmax = (unsigned)T;
        dmax = (unsigned)D;
    }
    if (b == bk.nbricks) dcount[b] = 0;
    tmax = __reduce_max_sync(0xffffffffu, tmax);
    dmax = __reduce_max_sync(0xffffffffu, dmax);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(stats, tmax);
        atomicMax(stats + 1, dmax);
    }
}

// the largest source staging of any brick over every source array, as the
// staged-record capacity, if it fits the shared memory of a block
constexpr int kBrickSmemLimit = 200 * 1024;

// Shared-memory layout of a pass over destination array D from source S.
int brick_layout(const sph_ctx *ctx, const ArraySnap &S, bool rates, bool cells, BrickSmem *sm,
                 size_t *bytes) {
    const BrickGeom &bk = ctx->bricks;
    const Grid &g = ctx->grid;
    const int lx = bk.bx + 2 * g.kx, ry = bk.by + 2 * g.ky, rz = bk.bz + 2 * g.kz;
    const int nr = ry * rz;
    const int ndr = bk.by * bk.bz;
    // tables (ints): rlo[nr], roff[nr + 1], dlo[ndr], doff[ndr + 1], and for
    // a list build scell[nr (lx + 1)]
    const size_t ncell = cells ? (size_t)nr * (lx + 1) : 0;
    const size_t tables = sizeof(int) * ((size_t)nr + nr + 1 + ndr + ndr + 1 + ncell);
    const size_t rec = rates ? (16 + 16 + 8) : 16;
    // the staged records and the padding record after them
    size_t cap = (size_t)std::max(S.b_tmax, 0) + 1;
    // environment SPH_BRICK_UNSTAGED=1 reads every record from global memory
    // (the path of bricks too populous for shared memory), to test it on
    // small sets
    static int unstaged = -1;
    if (unstaged < 0) {
        const char *e = getenv("SPH_BRICK_UNSTAGED");
        unstaged = (e && atoi(e) > 0) ? 1 : 0;
    }
    bool staged = !unstaged && tables + cap * rec + 64 <= (size_t)kBrickSmemLimit;
    if (!staged) cap = 0;
    size_t off = 0;
    sm->stage_cap = (int)cap;
    // position records, then (rates) velocity and state records
    off += cap * 16;
    sm->off_v = (int)off;
    if (rates) off += cap * 16;
    sm->off_s = (int)off;
    if (rates) off += cap * 8;
    off = (off + 15) & ~(size_t)15;
    sm->off_rlo = (int)off; off += sizeof(int) * nr;
    sm->off_roff = (int)off; off += sizeof(int) * (nr + 1);
    sm->off_dlo = (int)off; off += sizeof(int) * ndr;
    sm->off_doff = (int)off; off += sizeof(int) * (ndr + 1);
    sm->off_scell = (int)off; off += sizeof(int) * ncell;
    *bytes = off;
    return staged ? 1 : 0;
}

BrickRadius brick_radius(const sph_ctx *ctx) {
    const Grid &g = ctx->grid;
    BrickRadius r;
    const double radius = ctx->build_h * g.radius_scale;
    r.radius2 = radius * radius;
    const float r2 = (float)r.radius2;
    r.r2lo = r2 * (1.f - 1e-5f);
    r.r2hi = r2 * (1.f + 1e-5f);
    r.r2list = 0.f;
    if (g.skin > 0.f) {
        const float rl = (float)radius + g.skin;
        r.r2list = rl * rl * (1.f + 2e-5f);
    }
    return r;
}

BrickSrcDev make_bsrc(const ArraySnap &S) {
    BrickSrcDev s;
    s.pm = S.pm; s.velh = S.velh; s.st = S.st; s.scx = S.scx;
    s.cstart = S.cstart; s.perm = S.perm;
    s.x = S.view.x; s.y = S.view.y; s.z = S.view.z;
    return s;
}

BrickDstDev make_bdst(const ArraySnap &D) {
    BrickDstDev d;
    d.pm = D.pm; d.velh = D.velh; d.st = D.st; d.scx = D.scx;
    d.cstart = D.cstart; d.perm = D.perm; d.bdst = D.bdst;
    d.tag = D.view.tag;
    d.x = D.view.x; d.y = D.view.y; d.z = D.view.z; d.h = D.view.h;
    d.u = D.view.u; d.v = D.view.v; d.w = D.view.w;
    d.p = D.view.p; d.cs = D.view.cs;
    return d;
}

// Threads per block: the largest brick population rounded to warps, at
// most 320 (three blocks of 64-register threads per SM); a brick with more
// destinations takes them in rounds.
int brick_threads(const ArraySnap &D) {
    // environment SPH_BRICK_MAX_THREADS: another ceiling (a multiple of 32
    // up to 512), to measure it
    static int ceiling = -1;
    if (ceiling < 0) {
        const char *e = getenv("SPH_BRICK_MAX_THREADS");
        const int v = e ? atoi(e) : 0;
        ceiling = (v >= 64 && v <= kBrickMaxThreads && v % 32 == 0) ? v : 320;
    }
    const int want = (std::max(D.b_dmax, 1) + 31) / 32 * 32;
    return std::min(std::max(want, 64), ceiling);
}

template <class Kern>
int allow_smem(Kern *k, size_t bytes) {
    // raise each kernel's dynamic shared-memory limit to the largest layout,
    // once per kernel and device
    static std::mutex mu;
    static std::vector<std::pair<const void *, int>> done;
    if (bytes <= 48 * 1024) return SPH_OK;
    int dev = 0;
    SPH_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    for (const auto &d : done)
        if (d.first == (const void *)k && d.second == dev) return SPH_OK;
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               kBrickSmemLimit);
    if (e != cudaSuccess) return cuda_check(e, "cudaFuncSetAttribute (brick shared memory)");
    done.emplace_back((const void *)k, dev);
    return SPH_OK;
}

}  // namespace

// Brick geometry of the current grid: edge lengths (cells) per stencil
// half-width, chosen so a brick holds a few hundred destinations and its
// staging ~5-8 times as many sources.
void brick_geometry(sph_ctx *ctx) {
    const Grid &g = ctx->grid;
    BrickGeom &bk = ctx->bricks;
    const int K = g.kx;
    // environment SPH_BRICK_EDGE: the brick edge in cells (3D), to measure
    // other brick sizes
    static int edge = -1;
    // environment SPH_BRICK_SHAPE=bx,by,bz: a 3D brick shape, to measure it
    static int shape[3] = {0, 0, 0};
    if (edge < 0) {
        const char *e = getenv("SPH_BRICK_EDGE");
        edge = e ? std::max(1, atoi(e)) : 0;
        const char *sh = getenv("SPH_BRICK_SHAPE");
        int a = 0, b = 0, c = 0;
        if (sh && sscanf(sh, "%d,%d,%d", &a, &b, &c) == 3 && a > 0 && b > 0 && c > 0 && a <= 16 &&
            b <= 16 && c <= 16) {
            shape[0] = a; shape[1] = b; shape[2] = c;
        }
    }
    if (g.kz > 0) {
        const int e = edge > 0 ? edge : (K == 1 ? 3 : (K == 2 ? 5 : 8));
        bk.bx = bk.by = bk.bz = e;
        // stencil half-width 2: 6 x 5 x 5 cells (1 M-particle lattice, rates
        // pass 0.276 ms against 0.283 ms with 5^3 cells)
        if (K == 2 && edge <= 0) bk.bx = 6;
        if (shape[0] > 0) {
            bk.bx = shape[0]; bk.by = shape[1]; bk.bz = shape[2];
        }
    } else if (g.ky > 0) {
        const int e = K == 1 ? 8 : (K == 2 ? 12 : 16);
        bk.bx = bk.by = e;
        bk.bz = 1;
    } else {
        bk.bx = 64;
        bk.by = bk.bz = 1;
    }
    bk.nbx = (g.nx + bk.bx - 1) / bk.bx;
    bk.nby = (g.ny + bk.by - 1) / bk.by;
    bk.nbz = (g.nz + bk.bz - 1) / bk.bz;
    bk.nbricks = (int64_t)bk.nbx * bk.nby * bk.nbz;
}

// Per-array brick tables for the current build (queued on the context's
// stream); the statistics land in stats[2 a], stats[2 a + 1].
int brick_tables(sph_ctx *ctx, int a, unsigned *stats) {
    ArraySnap &A = ctx->arrays[a];
    const BrickGeom &bk = ctx->bricks;
    const int64_t need = bk.nbricks + 1;
    if (need > A.bdst_cap || !A.bdst) {
        cudaFree(A.bdst);
        A.bdst = nullptr;
        SPH_CUDA(cudaMalloc(&A.bdst, sizeof(int) * need));
        A.bdst_cap = need;
    }
    const int th = 128;
    const int blocks = (int)((need + th - 1) / th);
    k_brick_tables<<<blocks, th, 0, ctx->stream>>>(ctx->grid, bk, A.cstart, A.bdst, stats);
    count_launch();
    SPH_LAUNCH_CHECK("k_brick_tables");
    return scan_exclusive(ctx, A.bdst, need);
}

bool brick_density_eligible(const sph_ctx *ctx, int dst, const int *srcs, int nsrc,
                            const sph_density_params *prm) {
    const Grid &g = ctx->grid;
    if (!ctx->bricks_on || !ctx->bricks_ready || nsrc != 1 || !g.uniform_h || g.periodic ||
        g.symmetric || prm->h0 != 0.0)
        return false;
    const ArraySnap &S = ctx->arrays[srcs[0]];
    const ArraySnap &D = ctx->arrays[dst];
    return S.n > 0 && D.n > 0 && S.b_tmax < 65535;
}

bool brick_rates_eligible(const sph_ctx *ctx, int dst, const sph_source_term *terms, int nterms,
                          const sph_rates_params *prm) {
    const Grid &g = ctx->grid;
    if (!ctx->bricks_on || !ctx->bricks_ready || nterms != 1 || !g.uniform_h || g.periodic ||
        g.symmetric || prm->drho_out != nullptr)
        return false;
    const uint32_t f = terms[0].flags;
    if (f != (SPH_TERM_PGRAD | SPH_TERM_AVISC) && f != (SPH_TERM_PGRAD | SPH_TERM_AVISC | SPH_TERM_XSPH))
        return false;
    const ArraySnap &S = ctx->arrays[terms[0].src];
    const ArraySnap &D = ctx->arrays[dst];
    return S.n > 0 && D.n > 0 && S.b_tmax < 65535;
}

// Density pass (and, with build, the list build) of destination dst among
// source src; write_out = 0 builds the list only.
int brick_density(sph_ctx *ctx, int dst, int src, NbrList &L, bool build, bool write_out,
                  const sph_density_params *prm, double *rho, double *p, double *cs,
                  float4 *st_out) {
    ArraySnap &D = ctx->arrays[dst];
    ArraySnap &S = ctx->arrays[src];
    BrickDensityArgs a{};
    a.g = ctx->grid;
    a.bk = ctx->bricks;
    a.rad = brick_radius(ctx);
    a.d = make_bdst(D);
    a.s = make_bsrc(S);
    size_t bytes = 0;
    const bool staged = brick_layout(ctx, S, false, build, &a.sm, &bytes) != 0;
    a.nbr = L.nbr16;
    a.cnt = L.cnt;
    a.maxcnt = L.maxcnt;
    a.cap = L.cap;
    a.build = build ? 1 : 0;
    a.write_out = write_out ? 1 : 0;
    if (prm) {
        a.dim = prm->dim;
        a.tait = prm->tait;
        a.co = (float)prm->co; a.ro = (float)prm->ro; a.gamma = (float)prm->gamma;
    } else {
        a.dim = ctx->dim;
    }
    a.rho_out = rho; a.p_out = p; a.cs_out = cs;
    a.st_out = st_out;
    a.gate = ctx->gate;
    if (D.n == 0) return SPH_OK;
    const int nt = brick_threads(D);
    const int blocks = (int)ctx->bricks.nbricks;
    const int K = ctx->grid.kx;
#define BDL2(K_, B_, S_)                                                                  \
    do {                                                                                  \
        int rc_ = allow_smem(k_bdensity<K_, B_, S_>, bytes);                              \
        if (rc_) return rc_;                                                              \
        k_bdensity<K_, B_, S_><<<blocks, nt, bytes, ctx->stream>>>(a);                    \
    } while (0)
#define BDL1(K_, B_) do { if (staged) BDL2(K_, B_, true); else BDL2(K_, B_, false); } while (0)
#define BDL(K_) do { if (build) BDL1(K_, true); else BDL1(K_, false); } while (0)
    if (K == 1) BDL(1);
    else if (K == 2) BDL(2);
    else BDL(3);
#undef BDL
#undef BDL1
#undef BDL2
    count_launch();
    SPH_LAUNCH_CHECK("k_bdensity");
    return SPH_OK;
}

int brick_rates(sph_ctx *ctx, int dst, const sph_source_term &term, NbrList &L,
                const sph_rates_params *prm, double *const *acc, double *const *pos,
                int accumulate) {
    ArraySnap &D = ctx->arrays[dst];
    ArraySnap &S = ctx->arrays[term.src];
    BrickRatesArgs a{};
    a.g = ctx->grid;
    a.bk = ctx->bricks;
    a.rad = brick_radius(ctx);
    a.d = make_bdst(D);
    a.s = make_bsrc(S);
    size_t bytes = 0;
    const bool staged = brick_layout(ctx, S, true, false, &a.sm, &bytes) != 0;
    a.nbr = L.nbr16;
    a.cnt = L.cnt;
    a.cap = L.cap;
    a.dim = prm->dim;
    a.alpha = (float)term.alpha;
    a.beta = (float)term.beta;
    a.eta2 = (float)(term.eta * term.eta);
    a.eps = (float)term.eps;
    a.add_velocity = prm->add_velocity;
    a.add_gravity = prm->add_gravity;
    a.accumulate = accumulate;
    // alpha cs / 2 = (alpha / 2) f (2 (rho / 2))^3 with cs = f rho^3; the
    // environment setting SPH_BRICK_TWO_RECORDS=0 keeps three records
    static int two = -1;
    if (two < 0) {
        const char *e = getenv("SPH_BRICK_TWO_RECORDS");
        two = (e && atoi(e) == 0) ? 0 : 1;
    }
    a.tait_state = two && S.st_tait_f > 0.0 ? 1 : 0;
    a.tait_kc = (float)(4.0 * term.alpha * S.st_tait_f);
    a.gx = prm->gx; a.gy = prm->gy; a.gz = prm->gz;
    for (int c = 0; c < 3; ++c) {
        a.acc[c] = acc ? acc[c] : nullptr;
        a.pos[c] = pos ? pos[c] : nullptr;
    }
    a.gate = ctx->gate;
    if (D.n == 0) return SPH_OK;
    const bool xsph = (term.flags & SPH_TERM_XSPH) != 0;
    const int nt = brick_threads(D);
    const int blocks = (int)ctx->bricks.nbricks;
    const int K = ctx->grid.kx;
#define BRL2(K_, X_)                                                                      \
    do {                                                                                  \
        if (staged) {                                                                     \
            int rc_ = allow_smem(k_brates<K_, X_, true>, bytes);                          \
            if (rc_) return rc_;                                                          \
            k_brates<K_, X_, true><<<blocks, nt, bytes, ctx->stream>>>(a);                \
        } else {                                                                          \
            int rc_ = allow_smem(k_brates<K_, X_, false>, bytes);                         \
            if (rc_) return rc_;                                                          \
            k_brates<K_, X_, false><<<blocks, nt, bytes, ctx->stream>>>(a);               \
        }                                                                                 \
    } while (0)
#define BRL(K_) do { if (xsph) BRL2(K_, true); else BRL2(K_, false); } while (0)
    if (K == 1) BRL(1);
    else if (K == 2) BRL(2);
    else BRL(3);
#undef BRL
#undef BRL2
    count_launch();
    SPH_LAUNCH_CHECK("k_brates");
    return SPH_OK;
}

}  // namespace sphgb
