// Cell-list neighbour structure on a dense grid (sm_103a).
//
// Replaces the reference's CellManager (base/cell.pyx:757-1437: dict of
// IntPoint -> Cell with per-array index lists, rebinned particle by particle)
// and the FixedDestNbrParticleLocator cache (base/nnps.pyx:385-620: one
// LongArray of neighbour indices per destination).  Here a build is:
//
//   k_box       bounding box of all arrays in internal cells, max h, and the
//               reference's jump-tolerance check (cell.pyx:1422-1437)
//   k_keys      dense cell index per particle + per-cell counts (atomics)
//   scan        exclusive prefix of the counts -> cstart
//   k_scatter   counting-sort scatter (order within a cell arbitrary)
//   k_cellsort  per-cell insertion sort by original index (deterministic)
//   k_reorder   gather of the sorted FP32 snapshot (cell-local offsets)
//
// No per-destination neighbour list is stored: the pair kernels walk the
// stencil rows of the sorted arrays directly.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "sph_internal.cuh"

namespace sphgb {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int floor_cell(double x, double inv_cs) {
    return (int)floor(x * inv_cs);
}

// -------------------------------------------------------------------------
// bounding box / max h / jump check
// -------------------------------------------------------------------------
__global__ void k_box(sph_array_view a, double inv_cs, double inv_cs_ref, int *refcell,
                      int check_jump, int *box, unsigned long long *hmax, unsigned *err,
                      Grid pg) {
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX};
    int mx[3] = {INT_MIN, INT_MIN, INT_MIN};
    double hm = 0.0, hn = 1.0e308;
    bool jump = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double p[3] = {ld0(a.x, i), ld0(a.y, i), ld0(a.z, i)};
        const double pb[3] = {bin_x(pg, p[0]), p[1], p[2]};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int c = floor_cell(pb[d], inv_cs);
            mn[d] = min(mn[d], c);
            mx[d] = max(mx[d], c);
        }
        hm = fmax(hm, a.h[i]);
        hn = fmin(hn, a.h[i]);
        if (refcell) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                int c = floor_cell(p[d], inv_cs_ref);
                if (check_jump && abs(c - refcell[3 * i + d]) > 1) jump = true;
                refcell[3 * i + d] = c;
            }
        }
    }
    // warp, then block, then one set of atomics per block
    __shared__ int s_mn[3][32], s_mx[3][32];
    __shared__ double s_h[32], s_hn[32];
    __shared__ int s_j[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        mn[d] = __reduce_min_sync(0xffffffffu, mn[d]);
        mx[d] = __reduce_max_sync(0xffffffffu, mx[d]);
    }
    for (int off = 16; off > 0; off >>= 1) {
        hm = fmax(hm, __shfl_xor_sync(0xffffffffu, hm, off));
        hn = fmin(hn, __shfl_xor_sync(0xffffffffu, hn, off));
    }
    int anyjump = __any_sync(0xffffffffu, jump) ? 1 : 0;
    if (lane == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) { s_mn[d][wid] = mn[d]; s_mx[d][wid] = mx[d]; }
        s_h[wid] = hm;
        s_hn[wid] = hn;
        s_j[wid] = anyjump;
    }
    __syncthreads();
    if (wid == 0) {
        int a[3], b[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            a[d] = lane < nw ? s_mn[d][lane] : INT_MAX;
            b[d] = lane < nw ? s_mx[d][lane] : INT_MIN;
            a[d] = __reduce_min_sync(0xffffffffu, a[d]);
            b[d] = __reduce_max_sync(0xffffffffu, b[d]);
        }
        double hh = lane < nw ? s_h[lane] : 0.0;
        double hl = lane < nw ? s_hn[lane] : 1.0e308;
        for (int off = 16; off > 0; off >>= 1) {
            hh = fmax(hh, __shfl_xor_sync(0xffffffffu, hh, off));
            hl = fmin(hl, __shfl_xor_sync(0xffffffffu, hl, off));
        }
        int jj = __any_sync(0xffffffffu, lane < nw && s_j[lane]);
        if (lane == 0) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                atomicMin(&box[d], a[d]);
                atomicMax(&box[3 + d], b[d]);
            }
            atomicMax(hmax, (unsigned long long)__double_as_longlong(hh));
            atomicMin(hmax + 1, (unsigned long long)__double_as_longlong(hl));
            if (jj) atomicOr(err, SPH_EFLAG_JUMP);
        }
    }
}

__global__ void k_publish(const unsigned *src, unsigned *dst, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
    __threadfence_system();
}

__global__ void k_box_init(int *box, unsigned long long *hmax) {
    if (threadIdx.x < 3) {
        box[threadIdx.x] = INT_MAX;
        box[3 + threadIdx.x] = INT_MIN;
    }
    if (threadIdx.x == 0) {
        hmax[0] = 0ull;
        hmax[1] = (unsigned long long)__double_as_longlong(1.0e308);
    }
}

// -------------------------------------------------------------------------
// keys, counting sort
// -------------------------------------------------------------------------
__global__ void k_keys(sph_array_view a, Grid g, int *key, int *count) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int cx = bin_cell_x(g, bin_x(g, ld0(a.x, i)));
        int cy = floor_cell(ld0(a.y, i), g.inv_cs) - g.by0;
        int cz = floor_cell(ld0(a.z, i), g.inv_cs) - g.bz0;
        int k = cx + g.nx * (cy + g.ny * cz);
        key[i] = k;
        atomicAdd(&count[k], 1);
    }
}

// exclusive scan, 3 phases over tiles of kScanTile counts: tile totals
// (read only), exclusive scan of the totals, then each tile re-read, scanned
// and written with its offset.  Every thread moves one int4 per step, so a
// warp's accesses are 512 contiguous bytes.
constexpr int kScanV = 4;                                   // counts per thread per step
constexpr int kScanSteps = 8;
constexpr int kScanTile = kThreads * kScanV * kScanSteps;   // 8192 counts

__device__ __forceinline__ int block_exclusive_scan(int v, int *smem, int &total) {
    // warp inclusive scan
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) smem[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int nw = blockDim.x >> 5;
        int s = lane < nw ? smem[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, off);
            if (lane >= off) s += y;
        }
        if (lane < nw) smem[lane] = s;
    }
    __syncthreads();
    int warp_prefix = wid > 0 ? smem[wid - 1] : 0;
    total = smem[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

// the four counts of step st of this thread (0 past n)
__device__ __forceinline__ int4 scan_load(const int *data, int64_t n, int64_t i) {
    if (i + kScanV <= n) return *reinterpret_cast<const int4 *>(data + i);
    int4 v = make_int4(0, 0, 0, 0);
    if (i < n) v.x = data[i];
    if (i + 1 < n) v.y = data[i + 1];
    if (i + 2 < n) v.z = data[i + 2];
    return v;
}

__global__ void k_scan_reduce(const int *data, int64_t n, int *tile_tot) {
    __shared__ int smem[32];
    const int64_t base = blockIdx.x * (int64_t)kScanTile;
    int s = 0;
#pragma unroll
    for (int st = 0; st < kScanSteps; ++st) {
        const int4 v = scan_load(data, n, base + ((int64_t)st * kThreads + threadIdx.x) * kScanV);
        s += v.x + v.y + v.z + v.w;
    }
    int total;
    block_exclusive_scan(s, smem, total);
    if (threadIdx.x == 0) tile_tot[blockIdx.x] = total;
}

__global__ void k_scan_totals(int *tot, int64_t ntiles) {
    __shared__ int smem[32];
    int carry = 0;
    for (int64_t b = 0; b < ntiles; b += blockDim.x) {
        int64_t i = b + threadIdx.x;
        int v = i < ntiles ? tot[i] : 0;
        int total;
        int pre = block_exclusive_scan(v, smem, total);
        if (i < ntiles) tot[i] = pre + carry;
        carry += total;
    }
}

__global__ void k_scan_apply(int *data, int64_t n, const int *tile_off) {
    __shared__ int smem[32];
    const int64_t base = blockIdx.x * (int64_t)kScanTile;
    int carry = tile_off[blockIdx.x];
    for (int st = 0; st < kScanSteps; ++st) {
        const int64_t i = base + ((int64_t)st * kThreads + threadIdx.x) * kScanV;
        const int4 v = scan_load(data, n, i);
        int total;
        const int pre = carry + block_exclusive_scan(v.x + v.y + v.z + v.w, smem, total);
        const int4 o = make_int4(pre, pre + v.x, pre + v.x + v.y, pre + v.x + v.y + v.z);
        if (i + kScanV <= n) {
            *reinterpret_cast<int4 *>(data + i) = o;
        } else {
            if (i < n) data[i] = o.x;
            if (i + 1 < n) data[i + 1] = o.y;
            if (i + 2 < n) data[i + 2] = o.z;
        }
        carry += total;
    }
}

__global__ void k_scatter(int64_t n, const int *key, int *cursor, int *perm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int slot = atomicAdd(&cursor[key[i]], 1);
        perm[slot] = (int)i;
    }
}

__global__ void k_cellsort(int64_t ncells, const int *cstart, int *perm) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells;
         c += (int64_t)gridDim.x * blockDim.x) {
        int s = cstart[c], e = cstart[c + 1];
        for (int a = s + 1; a < e; ++a) {
            int v = perm[a];
            int b = a - 1;
            while (b >= s && perm[b] > v) {
                perm[b + 1] = perm[b];
                --b;
            }
            perm[b + 1] = v;
        }
    }
}

// -------------------------------------------------------------------------
// sorted snapshot
// -------------------------------------------------------------------------
__global__ void k_reorder(sph_array_view a, Grid g, const int *perm, const int *key, int *skey,
                          float *scx, float4 *velh, float4 *st, float4 *nrm, float4 *tan,
                          float4 *pm) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < a.n;
         s += (int64_t)gridDim.x * blockDim.x) {
        int i = perm[s];
        int k = key[i];
        skey[s] = k;
        int cx, cy, cz;
        decode_cell(g, k, cx, cy, cz);
        double ox = (double)(cx + g.bx0), oy = (double)(cy + g.by0), oz = (double)(cz + g.bz0);
        float xi = (float)fma(-ox, g.cs, bin_x(g, ld0(a.x, i)));
        float yi = (float)fma(-oy, g.cs, ld0(a.y, i));
        float zi = (float)fma(-oz, g.cs, ld0(a.z, i));
        scx[s] = (float)cx;
        velh[s] = make_float4((float)ld0(a.u, i), (float)ld0(a.v, i), (float)ld0(a.w, i),
                              (float)a.h[i]);
        float rho = (float)ld0(a.rho, i), p = (float)ld0(a.p, i), m = (float)a.m[i];
        st[s] = make_float4(rho, p / (rho * rho), (float)ld0(a.cs, i), m);
        pm[s] = make_float4(xi, yi, zi, m);
        if (nrm) {
            nrm[s] = make_float4((float)ld0(a.nx, i), (float)ld0(a.ny, i), (float)ld0(a.nz, i), 0.f);
            tan[s] = make_float4((float)ld0(a.tx, i), (float)ld0(a.ty, i), (float)ld0(a.tz, i), 0.f);
        }
    }
}

// Light refresh, in original particle order (coalesced FP64 reads, sorted
// slot from the inverse permutation of the last full build): the position
// and velocity records of the particle in the cell of that build (the
// state record waits for the next density pass, which rewrites it, or for
// k_state before a pass that reads it), the largest squared displacement
// from the build position, an h other than the build's uniform h, and the
// jump check against the previous update's cells.
// status[0] |= flags, status[1] = max(displacement^2 bits), and
// status[kStaleWord] = kStaleLists when some block saw a displacement of
// at least stale_thr^(1/2), an h change or a jump (the lists no longer hold
// every neighbour), or when a list of this build holds more neighbours than
// its capacity (the re-traversal that completes it needs the build's
// positions).
struct ListCaps {
    int n;                      // lists to check (0: none)
    int cap[kMaxListSlots];     // capacity, INT_MAX for a list of an older build
};

constexpr unsigned kLightHChanged = 1u << 8;

// The integer-operation conversions against the hardware's: input k is a
// hashed 64-bit pattern (every exponent and sign; NaN patterns skipped), and
// the first inputs are edge values (zero, extremes of the FP32 range, ties).
__device__ __forceinline__ unsigned long long selftest_bits(long long k) {
    unsigned long long z = (unsigned long long)k * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_selftest_conversions(long long n, unsigned long long *bad) {
    const double edge[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38,
                           1.1754943508222875e-38, 1.1754942106924411e-38, 1.401298464324817e-45,
                           1.0000000596046448, 1.0000001788139343, 0.5, 1e300, -1e-300,
                           8388608.5, 16777217.0};
    constexpr int NE = sizeof(edge) / sizeof(edge[0]);
    unsigned long long miss = 0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const unsigned long long b = selftest_bits(k);
        double x = k < NE ? edge[k] : __longlong_as_double((long long)b);
        if (x != x) x = __longlong_as_double((long long)(b & 0x800FFFFFFFFFFFFFull));
        if (__float_as_uint(d2f_rn(x)) != __float_as_uint(__double2float_rn(x))) ++miss;
        const int iv = (int)(unsigned)b;
        if (__double_as_longlong(i2d_exact(iv)) != __double_as_longlong(__int2double_rn(iv))) ++miss;
        // cell indices of positions in [-1000, 1000) at cell sizes 1e-3 .. 1
        const double pos = ((double)(b >> 11) * (1.0 / 9007199254740992.0)) * 2000.0 - 1000.0;
        const double inv = 1.0 / (1e-3 + (double)((b >> 3) & 1023) * 1e-3);
        if (floor_cell_screened(pos, inv, (float)inv) != (int)floor(pos * inv)) ++miss;
    }
    if (miss) atomicAdd(bad, miss);
}

// original -> sorted slot, and the build's position records in original
// order (so that a light refresh reads them with its other per-particle
// loads, not through the slot it has yet to load)
__global__ void k_invperm(int64_t n, const int *perm, const float4 *pm, int *inv, float4 *pm0) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int i = perm[s];
        inv[i] = (int)s;
        pm0[i] = pm[s];
    }
}

__global__ void __launch_bounds__(256, 5) k_light(sph_array_view a, Grid g, double inv_cs_ref, const int *inv,
                        const int *key, const float4 *pm0, float4 *velh,
                        float4 *nrm, float4 *tan, float4 *pm, int *refcell,
                        int check_jump,
                        double build_h, float stale_thr, const __grid_constant__ ListCaps caps,
                        unsigned *status, unsigned stale_bit) {
    float dm = 0.f;
    bool jump = false, hch = false;
    const float inv_ref_f = (float)inv_cs_ref;
    // list maxima: written by the passes before this launch
    if (blockIdx.x == 0 && threadIdx.x < caps.n &&
        (int)status[kListWord0 + threadIdx.x] > caps.cap[threadIdx.x]) {
        atomicOr(status + kStaleWord, kStaleLists);
        if (stale_bit) atomicOr(status + kStaleBitsWord, stale_bit);
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int s = inv[i];
        int cx, cy, cz;
        decode_cell(g, key[i], cx, cy, cz);
        const double px = ld0(a.x, i), py = ld0(a.y, i), pz = ld0(a.z, i);
        // the FP64 work of a refresh is the three offsets from the cell
        // origin; conversions and comparisons are done with integers
        const double ox = i2d_exact(cx + g.bx0), oy = i2d_exact(cy + g.by0), oz = i2d_exact(cz + g.bz0);
        const float xi = d2f_rn(fma(-ox, g.cs, bin_x(g, px)));
        const float yi = d2f_rn(fma(-oy, g.cs, py));
        const float zi = d2f_rn(fma(-oz, g.cs, pz));
        const float4 p0 = pm0[i];
        const float ddx = xi - p0.x, ddy = yi - p0.y, ddz = zi - p0.z;
        dm = fmaxf(dm, fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz)));
        const double h = a.h[i];
        if (__double_as_longlong(h) != __double_as_longlong(build_h)) hch = true;
        velh[s] = make_float4(d2f_rn(ld0(a.u, i)), d2f_rn(ld0(a.v, i)), d2f_rn(ld0(a.w, i)),
                              d2f_rn(h));
        pm[s] = make_float4(xi, yi, zi, d2f_rn(a.m[i]));
        if (nrm) {
            nrm[s] = make_float4((float)ld0(a.nx, i), (float)ld0(a.ny, i), (float)ld0(a.nz, i), 0.f);
            tan[s] = make_float4((float)ld0(a.tx, i), (float)ld0(a.ty, i), (float)ld0(a.tz, i), 0.f);
        }
        const double pp[3] = {px, py, pz};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            // the reference cell rarely changes between updates: store only
            // a change (no write-back of unchanged lines)
            const int c = floor_cell_screened(pp[d], inv_cs_ref, inv_ref_f);
            const int c0 = refcell[3 * i + d];
            if (check_jump && abs(c - c0) > 1) jump = true;
            if (c != c0) refcell[3 * i + d] = c;
        }
    }
    // warp, then block, then one atomic per block
    __shared__ float s_dm[32];
    __shared__ unsigned s_fl[32];
    for (int off = 16; off > 0; off >>= 1) dm = fmaxf(dm, __shfl_xor_sync(0xffffffffu, dm, off));
    const unsigned fl = (__any_sync(0xffffffffu, jump) ? SPH_EFLAG_JUMP : 0u) |
                        (__any_sync(0xffffffffu, hch) ? kLightHChanged : 0u);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
        s_dm[wid] = dm;
        s_fl[wid] = fl;
    }
    __syncthreads();
    if (wid == 0) {
        float b = lane < nw ? s_dm[lane] : 0.f;
        unsigned f = lane < nw ? s_fl[lane] : 0u;
        for (int off = 16; off > 0; off >>= 1) {
            b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, off));
            f |= __shfl_xor_sync(0xffffffffu, f, off);
        }
        if (lane == 0) {
            if (b > 0.f) atomicMax(status + 1, __float_as_uint(b));
            if (f) atomicOr(status, f);
            if (f || !(b < stale_thr)) {
                atomicOr(status + kStaleWord, kStaleLists);
                if (stale_bit) atomicOr(status + kStaleBitsWord, stale_bit);
            }
        }
    }
}

// State record (rho, p / rho^2, cs, m) of every particle in the slots of
// the last full build, after light refreshes that left it (in original
// order, as k_light).
__global__ void k_state(sph_array_view a, const int *inv, float4 *st) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float rho = (float)ld0(a.rho, i), p = (float)ld0(a.p, i);
        st[inv[i]] = make_float4(rho, p / (rho * rho), (float)ld0(a.cs, i), (float)a.m[i]);
    }
}

// -------------------------------------------------------------------------
// neighbour export (exact FP64 test; API / parity path, not the hot loop)
// -------------------------------------------------------------------------
template <bool FILL>
__global__ void k_nbr(sph_array_view d, sph_array_view s, Grid g, const int *dkey,
                      const int *scstart, const int *sperm, double radius_scale, int same,
                      int64_t *counts, const int64_t *offsets, int64_t *index) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int cx, cy, cz;
        decode_cell(g, dkey[i], cx, cy, cz);
        double px = ld0(d.x, i), py = ld0(d.y, i), pz = ld0(d.z, i);
        double radius = __dmul_rn(d.h[i], radius_scale);
        double r2 = __dmul_rn(radius, radius);
        int64_t cnt = 0;
        int64_t base = FILL ? offsets[i] : 0;
        for (int dz = -g.kz; dz <= g.kz; ++dz)
            for (int dy = -g.ky; dy <= g.ky; ++dy) {
                int64_t rowbase = (int64_t)g.nx * ((cy + dy) + (int64_t)g.ny * (cz + dz));
                // x cells [cx - kx, cx + kx]; on a periodic axis the cells past
                // either end wrap around and hold the images at x -+ period
                int pieces = 1, plo[3] = {cx - g.kx, 0, 0}, phi[3] = {cx + g.kx, 0, 0};
                double pshift[3] = {0.0, 0.0, 0.0};
                if (g.periodic) {
                    const int a0 = cx - g.kx, a1 = cx + g.kx;
                    pieces = 0;
                    if (a0 < 0) { plo[pieces] = a0 + g.nx; phi[pieces] = g.nx - 1; pshift[pieces++] = -g.plen; }
                    plo[pieces] = max(a0, 0); phi[pieces] = min(a1, g.nx - 1); pshift[pieces++] = 0.0;
                    if (a1 >= g.nx) { plo[pieces] = 0; phi[pieces] = a1 - g.nx; pshift[pieces++] = g.plen; }
                }
                for (int pc = 0; pc < pieces; ++pc) {
                int rs = scstart[rowbase + plo[pc]], re = scstart[rowbase + phi[pc] + 1];
                for (int t = rs; t < re; ++t) {
                    int j = sperm[t];
                    const double sx = pshift[pc] == 0.0 ? ld0(s.x, j) : __dadd_rn(ld0(s.x, j), pshift[pc]);
                    bool hit = exact_within(sx, ld0(s.y, j), ld0(s.z, j), px, py, pz, r2);
                    if (!hit && g.symmetric) {
                        // VarHNbrParticleLocator: i within the radius of j
                        const double rj = __dmul_rn(s.h[j], radius_scale);
                        hit = exact_within(px, py, pz, sx, ld0(s.y, j), ld0(s.z, j),
                                           __dmul_rn(rj, rj));
                    }
                    if (hit) {
                        if (FILL) index[base + cnt] = j;
                        ++cnt;
                    }
                }
                }
            }
        if (FILL) {
            // ascending, then self swapped with the last entry (the
            // reference's cache update, base/nnps.pyx:609-616)
            for (int64_t a2 = base + 1; a2 < base + cnt; ++a2) {
                int64_t v = index[a2];
                int64_t b = a2 - 1;
                while (b >= base && index[b] > v) {
                    index[b + 1] = index[b];
                    --b;
                }
                index[b + 1] = v;
            }
            if (same) {
                for (int64_t t = base; t + 1 < base + cnt; ++t)
                    if (index[t] == i) {
                        index[t] = index[base + cnt - 1];
                        index[base + cnt - 1] = i;
                        break;
                    }
            }
        } else {
            counts[i] = cnt;
        }
    }
}

template <class T>
int ensure(T **p, int64_t &cap, int64_t need) {
    if (need <= cap && *p) return SPH_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    int64_t c = std::max<int64_t>(need + need / 8, 256);
    SPH_CUDA(cudaMalloc((void **)p, sizeof(T) * c));
    cap = c;
    return SPH_OK;
}

int alloc_array(ArraySnap &A, int64_t n, bool nrm) {
    if (n <= A.cap && A.perm && (!nrm || A.nrm)) return SPH_OK;
    cudaFree(A.key); cudaFree(A.perm); cudaFree(A.skey);
    cudaFree(A.scx); cudaFree(A.pm); cudaFree(A.velh); cudaFree(A.st); cudaFree(A.nrm);
    cudaFree(A.tan);
    A.key = A.perm = A.skey = nullptr;
    A.scx = nullptr;
    A.pm = A.velh = A.st = A.nrm = A.tan = nullptr;
    int64_t c = std::max<int64_t>(n, 1);
    SPH_CUDA(cudaMalloc(&A.key, sizeof(int) * c));
    SPH_CUDA(cudaMalloc(&A.perm, sizeof(int) * c));
    SPH_CUDA(cudaMalloc(&A.skey, sizeof(int) * c));
    SPH_CUDA(cudaMalloc(&A.scx, sizeof(float) * c));
    SPH_CUDA(cudaMalloc(&A.pm, sizeof(float4) * c));
    SPH_CUDA(cudaMalloc(&A.velh, sizeof(float4) * c));
    SPH_CUDA(cudaMalloc(&A.st, sizeof(float4) * c));
    if (nrm) {
        SPH_CUDA(cudaMalloc(&A.nrm, sizeof(float4) * c));
        SPH_CUDA(cudaMalloc(&A.tan, sizeof(float4) * c));
    }
    A.cap = c;
    return SPH_OK;
}

}  // namespace

int publish_words(sph_ctx *ctx, const void *src, void *dst, int nwords) {
    if (nwords <= 0) return SPH_OK;
    k_publish<<<1, 128, 0, ctx->stream>>>((const unsigned *)src, (unsigned *)dst, nwords);
    count_launch();
    SPH_LAUNCH_CHECK("k_publish");
    return SPH_OK;
}

int scan_exclusive(sph_ctx *ctx, int *data, int64_t n) {
    int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    int rc = ensure(&ctx->scan_tmp, ctx->scan_tmp_cap, ntiles);
    if (rc) return rc;
    k_scan_reduce<<<(unsigned)ntiles, kThreads, 0, ctx->stream>>>(data, n, ctx->scan_tmp);
    k_scan_totals<<<1, 1024, 0, ctx->stream>>>(ctx->scan_tmp, ntiles);
    k_scan_apply<<<(unsigned)ntiles, kThreads, 0, ctx->stream>>>(data, n, ctx->scan_tmp);
    count_launch(3);
    SPH_LAUNCH_CHECK("scan");
    return SPH_OK;
}

void launch_counting_sort(cudaStream_t st, int64_t n, int64_t ncells, const int *key, int *cursor,
                          const int *cstart, int *perm) {
    k_scatter<<<grid_blocks(n, kThreads), kThreads, 0, st>>>(n, key, cursor, perm);
    k_cellsort<<<grid_blocks(ncells, kThreads), kThreads, 0, st>>>(ncells, cstart, perm);
    count_launch(2);
}

int grid_blocks(int64_t n, int threads, int per_sm) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    int64_t need = (n + threads - 1) / threads;
    int64_t cap = (int64_t)sms * per_sm;
    return (int)std::max<int64_t>(1, std::min(need, cap));
}

int nnps_build(sph_ctx *ctx, const sph_array_view *arrays, int narrays, double cell_size,
               double radius_scale, int subdiv, int check_jump) {
    if (narrays <= 0 || !arrays) return set_error(SPH_ERR_ARG, "nnps_build: no arrays");
    if (!(cell_size > 0)) return set_error(SPH_ERR_ARG, "nnps_build: cell_size must be > 0");
    if (subdiv < 1 || subdiv > 3) return set_error(SPH_ERR_ARG, "nnps_build: subdiv must be 1..3");
    cudaStream_t st = ctx->stream;
    bool same_layout = (int)ctx->arrays.size() == narrays;
    if (same_layout)
        for (int a = 0; a < narrays; ++a)
            if (ctx->arrays[a].ref_n != arrays[a].n) same_layout = false;
    if ((int)ctx->arrays.size() != narrays) {
        free_lists(ctx);
        if ((int)ctx->arrays.size() < narrays) ctx->arrays.resize(narrays);
    }
    if (ctx->cell_size_ref != cell_size) same_layout = false;
    ctx->cell_size_ref = cell_size;

    // with a list skin the grid cell is the reference cell grown by the skin
    // fraction, so the stencil of the subdivision still covers the list radius
    const double skin_frac = ctx->skin_frac > 0.0 ? ctx->skin_frac : 0.0;
    double cs = cell_size * (1.0 + skin_frac) / subdiv;
    // periodic x: the period holds a whole number of (slightly larger) cells
    Grid pg;
    int pnx = 0;
    if (ctx->periodic) {
        const double plen = ctx->pxmax - ctx->pxmin;
        pnx = (int)std::floor(plen / cs);
        if (pnx < 1) return set_error(SPH_ERR_NOTSUP, "nnps_build: periodic domain shorter than a cell");
        cs = plen / pnx;
        pg.periodic = 1;
        pg.pxmin = ctx->pxmin;
        pg.plen = plen;
    }
    const double inv_cs = 1.0 / cs;
    const double inv_cs_ref = 1.0 / cell_size;

    k_box_init<<<1, 32, 0, st>>>(ctx->d_box, ctx->d_hmax);
    count_launch();
    SPH_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), st));
    for (int a = 0; a < narrays; ++a) {
        ArraySnap &A = ctx->arrays[a];
        const sph_array_view &v = arrays[a];
        if (v.n < 0 || (v.n > 0 && (!v.x || !v.h || !v.m)))
            return set_error(SPH_ERR_ARG, "nnps_build: array needs x, h and m");
        if (v.n >= (int64_t)INT32_MAX) return set_error(SPH_ERR_ARG, "nnps_build: array too large");
        int64_t rn = A.ref_n;
        if (rn != v.n) {
            cudaFree(A.refcell);
            A.refcell = nullptr;
            SPH_CUDA(cudaMalloc(&A.refcell, sizeof(int) * 3 * std::max<int64_t>(v.n, 1)));
            A.ref_n = v.n;
        }
        if (v.n == 0) continue;
        int jb = (check_jump && same_layout) ? 1 : 0;
        k_box<<<grid_blocks(v.n, kThreads, 8), kThreads, 0, st>>>(v, inv_cs, inv_cs_ref, A.refcell, jb,
                                                               ctx->d_box, ctx->d_hmax, ctx->d_err,
                                                               pg);
        count_launch();
        SPH_LAUNCH_CHECK("k_box");
    }
    {
        int rcp = publish_words(ctx, ctx->d_box, ctx->hd_box, 6);
        if (!rcp) rcp = publish_words(ctx, ctx->d_hmax, ctx->hd_box + 6, 4);   // hmax, hmin
        if (rcp) return rcp;
    }
    {
        const int rcm = list_maxima_async(ctx);   // with the error word
        if (rcm) return rcm;
    }
    SPH_CUDA(cudaStreamSynchronize(st));
    list_maxima_collect(ctx);
    unsigned err = ctx->h_status[0];
    if (err & SPH_EFLAG_JUMP) {
        ctx->built = false;
        return set_error(SPH_ERR_JUMP, "Particle moved by more than one cell width");
    }
    int64_t total_n = 0;
    for (int a = 0; a < narrays; ++a) total_n += arrays[a].n;
    if (total_n == 0) return set_error(SPH_ERR_ARG, "nnps_build: no particles");

    double hmax, hmin;
    memcpy(&hmax, ctx->h_box + 6, sizeof(hmax));
    memcpy(&hmin, ctx->h_box + 8, sizeof(hmin));
    Grid g;
    g.periodic = pg.periodic;
    g.pxmin = pg.pxmin;
    g.plen = pg.plen;
    g.cs = cs;
    g.inv_cs = inv_cs;
    g.cs_f = (float)cs;
    g.radius_scale = radius_scale;
    g.uniform_h = (hmin == hmax) ? 1 : 0;
    g.h_uniform = (float)hmax;
    const double skin = skin_frac * radius_scale * hmax;
    g.skin = (float)skin;
    g.symmetric = ctx->symmetric;
    g.reach2 = (float)((radius_scale * hmax + skin) * (radius_scale * hmax + skin) * (1.0 + 1e-4));
    // the list radius over the grid cell, (rs hmax (1 + f)) / (cell (1 + f) / subdiv),
    // is the subdivision itself when cell = rs hmax; the margin absorbs rounding
    int k = (int)std::ceil((radius_scale * hmax + skin) * inv_cs - 1e-7);
    if (k < 1) k = 1;
    if (k > 3)
        return set_error(SPH_ERR_NOTSUP,
                         "nnps_build: search radius spans more than 3 cells (cell size too small)");
    int mn[3], mx[3];
    for (int d = 0; d < 3; ++d) { mn[d] = ctx->h_box[d]; mx[d] = ctx->h_box[3 + d]; }
    g.kx = k;
    g.ky = (mx[1] > mn[1]) ? k : 0;
    g.kz = (mx[2] > mn[2]) ? k : 0;
    g.bx0 = mn[0] - g.kx;
    g.by0 = mn[1] - g.ky;
    g.bz0 = mn[2] - g.kz;
    int64_t nx = (int64_t)mx[0] - mn[0] + 1 + 2 * g.kx;
    if (g.periodic) {
        // the grid is the period: a stencil row wraps at most once
        if (pnx < 2 * k + 1)
            return set_error(SPH_ERR_NOTSUP,
                             "nnps_build: periodic domain narrower than the neighbour stencil");
        g.bx0 = 0;
        nx = pnx;
    }
    int64_t ny = (int64_t)mx[1] - mn[1] + 1 + 2 * g.ky;
    int64_t nz = (int64_t)mx[2] - mn[2] + 1 + 2 * g.kz;
    const int64_t kMaxCells = (int64_t)1 << 27;
    if (nx * ny > kMaxCells || nx * ny * nz > kMaxCells)
        return set_error(SPH_ERR_GRID,
                         "nnps_build: particle extent needs more than 2^27 grid cells");
    if (nx > (1 << 24))
        return set_error(SPH_ERR_GRID, "nnps_build: more than 2^24 cells along x");
    g.nx = (int)nx; g.ny = (int)ny; g.nz = (int)nz;
    g.ncells = nx * ny * nz;
    ctx->grid = g;
    // stencil half-width 2 with more source particles than three 3-bit
    // offset fields leave slot bits for: base-5 offsets (environment
    // SPH_WIDE_CODES=1 forces them, to test them on small sets)
    {
        static int force = -1;
        if (force < 0) {
            const char *e = getenv("SPH_WIDE_CODES");
            force = (e && atoi(e) > 0) ? 1 : 0;
        }
        int64_t nmax = 0;
        for (int a = 0; a < narrays; ++a) nmax = std::max<int64_t>(nmax, arrays[a].n);
        ctx->wide_codes = k == 2 && (force || nmax >= ((int64_t)1 << 23));
    }

    for (int a = 0; a < narrays; ++a) {
        ArraySnap &A = ctx->arrays[a];
        const sph_array_view &v = arrays[a];
        A.view = v;
        A.n = v.n;
        A.has_nrm = v.nx || v.ny || v.nz;
        int rc = alloc_array(A, v.n, A.has_nrm);
        if (rc) return rc;
        if (g.ncells + 1 > A.cell_cap || !A.cstart) {
            cudaFree(A.cstart);
            cudaFree(A.cursor);
            A.cstart = A.cursor = nullptr;
            int64_t c = g.ncells + 1 + (g.ncells + 1) / 4;
            SPH_CUDA(cudaMalloc(&A.cstart, sizeof(int) * c));
            SPH_CUDA(cudaMalloc(&A.cursor, sizeof(int) * c));
            A.cell_cap = c;
        }
        SPH_CUDA(cudaMemsetAsync(A.cstart, 0, sizeof(int) * (g.ncells + 1), st));
        if (v.n > 0) {
            int nb = grid_blocks(v.n, kThreads);
            k_keys<<<nb, kThreads, 0, st>>>(v, g, A.key, A.cstart);
            count_launch();
            SPH_LAUNCH_CHECK("k_keys");
        }
        rc = scan_exclusive(ctx, A.cstart, g.ncells + 1);
        if (rc) return rc;
        if (v.n > 0) {
            SPH_CUDA(cudaMemcpyAsync(A.cursor, A.cstart, sizeof(int) * g.ncells,
                                     cudaMemcpyDeviceToDevice, st));
            int nb = grid_blocks(v.n, kThreads);
            k_scatter<<<nb, kThreads, 0, st>>>(v.n, A.key, A.cursor, A.perm);
            k_cellsort<<<grid_blocks(g.ncells, kThreads), kThreads, 0, st>>>(g.ncells, A.cstart, A.perm);
            k_reorder<<<nb, kThreads, 0, st>>>(v, g, A.perm, A.key, A.skey, A.scx, A.velh, A.st,
                                               A.has_nrm ? A.nrm : nullptr,
                                               A.has_nrm ? A.tan : nullptr, A.pm);
            count_launch(3);
            SPH_LAUNCH_CHECK("nnps sort/reorder");
            A.st_fresh = true;
            A.st_tait_f = 0.0;
            if (g.skin > 0.f) {
                if (A.pm0_cap < v.n) {
                    cudaFree(A.pm0);
                    cudaFree(A.inv);
                    A.pm0 = nullptr;
                    A.inv = nullptr;
                    SPH_CUDA(cudaMalloc(&A.pm0, sizeof(float4) * v.n));
                    SPH_CUDA(cudaMalloc(&A.inv, sizeof(int) * v.n));
                    A.pm0_cap = v.n;
                }
                k_invperm<<<grid_blocks(v.n, kThreads), kThreads, 0, st>>>(v.n, A.perm, A.pm, A.inv,
                                                                           A.pm0);
                count_launch();
                SPH_LAUNCH_CHECK("k_invperm");
            }
        }
    }
    ctx->built = true;
    ctx->build_id += 1;
    ctx->build_radius_scale = radius_scale;
    ctx->build_subdiv = subdiv;
    ctx->build_h = g.uniform_h ? hmax : 0.0;
    ctx->n_full += 1;
    // brick tables of the brick-staged pair passes (uniform h, no periodic
    // axis or symmetric relation): their largest populations size the
    // launches, so they are read back once per full build
    ctx->bricks_ready = false;
    if (ctx->bricks_on && g.uniform_h && !g.periodic && !g.symmetric &&
        narrays <= kMaxBrickArrays) {
        brick_geometry(ctx);
        SPH_CUDA(cudaMemsetAsync(ctx->d_bstats, 0, 2 * narrays * sizeof(unsigned), st));
        for (int a = 0; a < narrays; ++a) {
            if (arrays[a].n == 0) continue;
            const int rc = brick_tables(ctx, a, ctx->d_bstats + 2 * a);
            if (rc) return rc;
        }
        const int rp = publish_words(ctx, ctx->d_bstats, ctx->hd_bstats, 2 * narrays);
        if (rp) return rp;
        SPH_CUDA(cudaStreamSynchronize(st));
        for (int a = 0; a < narrays; ++a) {
            ArraySnap &A = ctx->arrays[a];
            A.b_tmax = arrays[a].n > 0 ? (int)ctx->h_bstats[2 * a] : 0;
            A.b_dmax = arrays[a].n > 0 ? (int)ctx->h_bstats[2 * a + 1] : 0;
        }
        ctx->bricks_ready = true;
    }
    return SPH_OK;
}

// Refresh the sorted snapshot of moved particles in the order of the last
// full build (the skin keeps the neighbour lists of that build valid while
// every particle stays within half the skin of its build position), with
// the reference's jump check (cell.pyx:1422-1437) against the previous
// update.  Falls back to a full build when a particle moved too far, an h
// changed, the array layout changed, or a list overflowed its capacity.
namespace {

// Verdict of a light refresh from its status block on the host: an error
// for a jump; *stale: the lists miss neighbours or a list outgrew its
// capacity (the word the gated passes test); *overflow: the host's own
// reading of the capacities (implies *stale, which k_light also sets).
int light_verdict(sph_ctx *ctx, bool *stale, bool *overflow) {
    *overflow = false;
    for (int i = 0; i < (int)ctx->lists.size() && i < kMaxListSlots; ++i) {
        const NbrList &L = ctx->lists[i];
        if (L.maxcnt && L.build == ctx->build_id && (int)ctx->h_status[kListWord0 + i] > L.cap)
            *overflow = true;
    }
    *stale = (ctx->h_status[kStaleWord] & kStaleLists) != 0;
    if (ctx->h_status[0] & SPH_EFLAG_JUMP) {
        ctx->built = false;
        return set_error(SPH_ERR_JUMP, "Particle moved by more than one cell width");
    }
    return SPH_OK;
}

}  // namespace

int resolve_pending(sph_ctx *ctx, bool *rebuilt) {
    *rebuilt = false;
    if (!ctx->pending) return SPH_OK;
    ctx->pending = false;
    SPH_CUDA(cudaEventSynchronize(ctx->pending_event));
    list_maxima_collect(ctx);
    bool stale, overflow;
    const int rc = light_verdict(ctx, &stale, &overflow);
    if (rc) return rc;
    if (stale) {
        // the refcells already hold the update's cells
        ctx->n_deferred_stale += 1;
        const int rb = nnps_build(ctx, ctx->pending_views.data(), (int)ctx->pending_views.size(),
                                  ctx->pending_cell_size, ctx->pending_radius_scale,
                                  ctx->pending_subdiv, 0);
        if (rb) return rb;
        *rebuilt = true;
        return SPH_OK;
    }
    // the gated pass has run on valid lists
    ctx->n_light += 1;
    return SPH_OK;
}

int nnps_update(sph_ctx *ctx, const sph_array_view *arrays, int narrays, double cell_size,
                double radius_scale, int subdiv, int check_jump, int *rebuilt) {
    if (rebuilt) *rebuilt = 1;
    {
        const int rc = resolve_pending(ctx);
        if (rc) return rc;
    }
    bool light = ctx->built && ctx->grid.skin > 0.f &&
                 narrays == (int)ctx->arrays.size() &&
                 cell_size == ctx->cell_size_ref && radius_scale == ctx->build_radius_scale &&
                 subdiv == ctx->build_subdiv && arrays != nullptr &&
                 ctx->build_h > 0.0 && (int)ctx->lists.size() <= kMaxListSlots &&
                 ctx->grid.symmetric == ctx->symmetric && ctx->grid.periodic == ctx->periodic;
    for (int a = 0; light && a < narrays; ++a) {
        const ArraySnap &A = ctx->arrays[a];
        const sph_array_view &v = arrays[a];
        if (v.n != A.n || v.n != A.ref_n || (v.n > 0 && (!v.x || !v.h || !v.m)) ||
            (bool)(v.nx || v.ny || v.nz) != A.has_nrm || (v.n > 0 && (!A.pm0 || !A.inv)))
            light = false;
    }
    if (!light) {
        // a full build needs the host: no step graph for this build
        if (ctx->capturing) {
            ctx->capture_failed = true;
            ctx->capture_fail_site = 1;   // the update needs a full build
            return SPH_OK;
        }
        return nnps_build(ctx, arrays, narrays, cell_size, radius_scale, subdiv, check_jump);
    }

    cudaStream_t st = ctx->stream;
    // error word, displacement, stale flag (a captured step clears them once,
    // at its start, so that a stale refresh gates the rest of the step)
    if (!ctx->capturing) SPH_CUDA(cudaMemsetAsync(ctx->d_status, 0, 3 * sizeof(unsigned), st));
    const double inv_cs_ref = 1.0 / cell_size;
    const float half = 0.5f * ctx->grid.skin;
    const float stale_thr = half * half * (1.f - 1e-4f);
    ListCaps caps;
    caps.n = std::min((int)ctx->lists.size(), kMaxListSlots);
    for (int i = 0; i < caps.n; ++i) {
        const NbrList &L = ctx->lists[i];
        caps.cap[i] = (L.maxcnt && L.build == ctx->build_id) ? L.cap : INT_MAX;
    }
    for (int a = 0; a < narrays; ++a) {
        ArraySnap &A = ctx->arrays[a];
        const sph_array_view &v = arrays[a];
        if (v.n == 0) continue;
        // one thread per particle (more loads in flight than a grid-stride
        // loop over a resident grid: 55 against 61 us at 1 M particles)
        k_light<<<grid_blocks(v.n, kThreads, 64), kThreads, 0, st>>>(
            v, ctx->grid, inv_cs_ref, A.inv, A.key, A.pm0, A.velh,
            A.has_nrm ? A.nrm : nullptr, A.has_nrm ? A.tan : nullptr, A.pm, A.refcell, check_jump,
            ctx->build_h, stale_thr, caps, ctx->d_status, ctx->capture_stale_bit);
        caps.n = 0;   // checked once
        A.st_fresh = false;
        count_launch();
        SPH_LAUNCH_CHECK("k_light");
    }
    for (int a = 0; a < narrays; ++a) ctx->arrays[a].view = arrays[a];
    if (ctx->capturing) {
        // the graph publishes the status block once, at the end of the step
        if (rebuilt) *rebuilt = 0;
        return SPH_OK;
    }
    {
        const int rcm = list_maxima_async(ctx);   // with the error word and displacement
        if (rcm) return rcm;
    }
    if (ctx->deferred) {
        SPH_CUDA(cudaEventRecord(ctx->pending_event, st));
        ctx->pending = true;
        ctx->pending_views.assign(arrays, arrays + narrays);
        ctx->pending_cell_size = cell_size;
        ctx->pending_radius_scale = radius_scale;
        ctx->pending_subdiv = subdiv;
        ctx->n_deferred += 1;
        if (rebuilt) *rebuilt = 0;
        return SPH_OK;
    }
    SPH_CUDA(cudaStreamSynchronize(st));
    list_maxima_collect(ctx);
    // a list that overflowed its capacity completes itself by re-traversal in
    // the order of its build: it needs the build's positions
    bool stale, overflow;
    const int rc = light_verdict(ctx, &stale, &overflow);
    if (rc) return rc;
    if (stale || overflow) {
        // too far for the lists: the refcells already hold this update's cells
        return nnps_build(ctx, arrays, narrays, cell_size, radius_scale, subdiv, 0);
    }
    ctx->n_light += 1;
    if (rebuilt) *rebuilt = 0;
    return SPH_OK;
}

int ensure_state(sph_ctx *ctx, int a) {
    ArraySnap &A = ctx->arrays[a];
    if (A.st_fresh) return SPH_OK;
    A.st_fresh = true;
    A.st_tait_f = 0.0;
    if (A.n == 0) return SPH_OK;
    if (!A.inv) return set_error(SPH_ERR_STATE, "state refresh without a light-refresh order");
    k_state<<<grid_blocks(A.n, kThreads, 64), kThreads, 0, ctx->stream>>>(A.view, A.inv, A.st);
    count_launch();
    SPH_LAUNCH_CHECK("k_state");
    return SPH_OK;
}

int refresh_state(sph_ctx *ctx, int a, const sph_array_view *view) {
    if (!ctx->built || a < 0 || a >= (int)ctx->arrays.size())
        return set_error(SPH_ERR_STATE, "refresh_state: no neighbour build for this array");
    ArraySnap &A = ctx->arrays[a];
    if (view->n != A.n)
        return set_error(SPH_ERR_STATE, "refresh_state: particle count changed; rebuild needed");
    bool nrm = view->nx || view->ny || view->nz;
    if (nrm && !A.nrm)
        return set_error(SPH_ERR_STATE, "refresh_state: normals added; rebuild needed");
    A.view = *view;
    A.has_nrm = nrm;
    A.st_fresh = true;
    A.st_tait_f = 0.0;
    if (A.n == 0) return SPH_OK;
    k_reorder<<<grid_blocks(A.n, kThreads), kThreads, 0, ctx->stream>>>(
        A.view, ctx->grid, A.perm, A.key, A.skey, A.scx, A.velh, A.st, nrm ? A.nrm : nullptr,
        nrm ? A.tan : nullptr, A.pm);
    count_launch();
    SPH_LAUNCH_CHECK("k_reorder (refresh)");
    return SPH_OK;
}

int nnps_count(sph_ctx *ctx, int dst, int src, double radius_scale, int64_t *counts) {
    if (!ctx->built || dst < 0 || src < 0 || dst >= (int)ctx->arrays.size() ||
        src >= (int)ctx->arrays.size())
        return set_error(SPH_ERR_STATE, "nnps_count: no neighbour build for these arrays");
    if (radius_scale > ctx->grid.radius_scale)
        return set_error(SPH_ERR_ARG, "nnps_count: radius_scale larger than the build's");
    ArraySnap &D = ctx->arrays[dst];
    ArraySnap &S = ctx->arrays[src];
    if (D.n == 0) return SPH_OK;
    k_nbr<false><<<grid_blocks(D.n, 128), 128, 0, ctx->stream>>>(
        D.view, S.view, ctx->grid, D.key, S.cstart, S.perm, radius_scale, dst == src,
        counts, nullptr, nullptr);
    count_launch();
    SPH_LAUNCH_CHECK("k_nbr count");
    return SPH_OK;
}

int nnps_fill(sph_ctx *ctx, int dst, int src, double radius_scale, const int64_t *offsets,
              int64_t *index) {
    if (!ctx->built || dst < 0 || src < 0 || dst >= (int)ctx->arrays.size() ||
        src >= (int)ctx->arrays.size())
        return set_error(SPH_ERR_STATE, "nnps_fill: no neighbour build for these arrays");
    if (radius_scale > ctx->grid.radius_scale)
        return set_error(SPH_ERR_ARG, "nnps_fill: radius_scale larger than the build's");
    ArraySnap &D = ctx->arrays[dst];
    ArraySnap &S = ctx->arrays[src];
    if (D.n == 0) return SPH_OK;
    k_nbr<true><<<grid_blocks(D.n, 128), 128, 0, ctx->stream>>>(
        D.view, S.view, ctx->grid, D.key, S.cstart, S.perm, radius_scale, dst == src,
        nullptr, offsets, index);
    count_launch();
    SPH_LAUNCH_CHECK("k_nbr fill");
    return SPH_OK;
}

int selftest_conversions(int64_t n, int64_t *mismatches) {
    if (n < 0 || !mismatches) return set_error(SPH_ERR_ARG, "selftest_conversions: bad argument");
    unsigned long long *d = nullptr;
    SPH_CUDA(cudaMalloc(&d, sizeof(unsigned long long)));
    cudaError_t e = cudaMemset(d, 0, sizeof(unsigned long long));
    if (e == cudaSuccess && n > 0) {
        k_selftest_conversions<<<grid_blocks(n, kThreads), kThreads>>>((long long)n, d);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_check(e, "selftest_conversions");
    *mismatches = (int64_t)h;
    return SPH_OK;
}

}  // namespace sphgb
