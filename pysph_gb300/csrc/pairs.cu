// Pair-loop kernels (sm_103a): neighbour lists, summation density (+ Tait)
// and the rates kernel (pressure gradient, Monaghan artificial viscosity,
// XSPH, Monaghan boundary force, with gravity / position stepping folded
// into the store).
//
// Replaces SPHCalc.sph -> SPHFunction.eval -> eval_single -> eval_nbr of the
// reference (sph/sph_calc.pyx:223-270, sph/sph_func.pyx:199-234,381-394,
// 466-484).  One thread owns one destination in cell-sorted order, so the
// threads of a warp walk the same stencil rows and their candidate loads
// are broadcasts.  Per evaluation:
//
//   k_nbrlist  tests the stencil candidates once (FP32 with an FP64 band
//              recheck, exact neighbour sets) and writes a k-major list of
//              (source slot | stencil offset code);
//   k_density  streams the list: sum m W, then Tait, per destination;
//   k_rates    streams the list: every rate term of the fused calcs.
//
// Sums are sequential per destination with Neumaier compensation, in the
// neighbour order of the list (stencil rows, ascending slot).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>

#include "sph_internal.cuh"

namespace sphgb {

namespace {

struct DestDev {
    const float4 *pm, *velh, *st;
    const int *skey, *perm;
    const int *sinst;    // batches: instance of each sorted slot
    const Grid *grids;   // batches: grid of each instance
    const int64_t *tag;
    const double *x, *y, *z, *u, *v, *w, *h, *p, *rho, *cs;
    int64_t n;
    int64_t s0;          // batches: first slot of the launch (slots [s0, n))
};

struct ListArgs {
    Grid g;
    DestDev d;
    SrcDev s;
    uint32_t *nbr;
    int *cnt;
    int *maxcnt;
    int64_t stride;
    int cap;
    const unsigned *gate;   // non-null: return at once if *gate (stale lists)
};

struct DensityArgs {
    Grid g;
    DestDev d;
    SrcDev s[SPH_MAX_SOURCES];
    int cap[SPH_MAX_SOURCES];
    int64_t stride[SPH_MAX_SOURCES];
    // per source: build the neighbour list while summing (list is stale)
    uint32_t *lnbr[SPH_MAX_SOURCES];
    int *lcnt[SPH_MAX_SOURCES];
    int *lmax[SPH_MAX_SOURCES];
    int nsrc;
    int dim;
    int tait;
    float co, ro, gamma;
    double *rho_out, *p_out, *cs_out;
    float4 *st_out; // sorted state of the destination (may be null)
    const unsigned *gate;
    float ih0;      // > 0: 1 / the fixed h of every pair (pilot density)
};

struct RatesArgs {
    Grid g;
    DestDev d;
    SrcDev s[SPH_MAX_SOURCES];
    int cap[SPH_MAX_SOURCES];
    int64_t stride[SPH_MAX_SOURCES];
    int nsrc;
    int dim;
    int add_velocity, add_gravity, accumulate;
    double gx, gy, gz;
    double *acc[3];
    double *pos[3];
    double *drho;
    const unsigned *gate;
    int vdiv;       // the drho sum is a velocity divergence: store -sum / rho_i
};

// Destination of thread slot s; false for a non-LocalReal particle.
__device__ __forceinline__ bool load_dest(const Grid &g, const DestDev &D, int s, DestPos &d) {
    const int orig = D.perm[s];
    d.orig = orig;
    if (D.tag != nullptr && D.tag[orig] != SPH_TAG_LOCAL_REAL) return false;
    const float4 p = D.pm[s];
    d.xi_x = p.x; d.xi_y = p.y; d.xi_z = p.z;
    decode_cell(g, D.skey[s], d.cx, d.cy, d.cz);
    const double radius = __dmul_rn(D.h[orig], g.radius_scale);
    d.radius2 = __dmul_rn(radius, radius);
    // FP32 copies by integer operations, bit-equal to the conversion: on
    // GB300 the narrow FP64 pipe executes the conversions too
    const float r2 = d2f_rn(d.radius2);
    d.r2lo = r2 * (1.f - 1e-5f);
    d.r2hi = r2 * (1.f + 1e-5f);
    d.r2list = 0.f;
    if (g.skin > 0.f) {
        const float rl = d2f_rn(radius) + g.skin;
        d.r2list = rl * rl * (1.f + 2e-5f);
    }
    return true;
}

// With a list skin the list holds sources up to the list radius: keep the
// neighbours (the FP32 band test, then the FP64 test of base/nnps.pyx:
// 337-353 inside the band).
template <bool EXT>
__device__ __forceinline__ bool listed_exact_test(const Grid &g, const SrcDev &S, const DestDev &D,
                                                  const DestPos &d, int j, float rx, float ry,
                                                  float rz) {
    const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
    if (r2 < d.r2lo) return true;
    bool hit = false;
    if (r2 <= d.r2hi) {
        const int oj = S.perm[j];
        const double xi = ld0(D.x, d.orig);
        hit = exact_within(EXT ? image_x(g, ld0(S.x, oj), xi, rx) : ld0(S.x, oj), ld0(S.y, oj),
                           ld0(S.z, oj), xi, ld0(D.y, d.orig), ld0(D.z, d.orig), d.radius2);
    }
    if (EXT && !hit && g.symmetric) {
        bool in_list;
        hit = reverse_within(g, S, j, r2, rx, D.x, D.y, D.z, d.orig, in_list);
    }
    return hit;
}

template <bool EXT>
__device__ __forceinline__ bool listed_exact(const Grid &g, const SrcDev &S, const DestDev &D,
                                             const DestPos &d, int j, float rx, float ry, float rz) {
    if (g.skin <= 0.f) return true;
    return listed_exact_test<EXT>(g, S, D, d, j, rx, ry, rz);
}

// grid of the destination in slot s
template <bool BATCH>
__device__ __forceinline__ const Grid &grid_of(const Grid &single, const DestDev &D, int s) {
    return BATCH ? D.grids[D.sinst[s]] : single;
}

// A pass launched after a deferred light refresh does nothing when the
// refresh found the lists stale (the host repeats it after a full build).
__device__ __forceinline__ bool gated_off(const unsigned *gate) {
    return gate != nullptr && __ldg(gate) != 0u;
}

// No per-neighbour data beyond the position record.
struct NoExtra {
    __device__ __forceinline__ int operator()(int) const { return 0; }
};

// Stream the neighbours of dest slot s from the list in batches of B.  The
// list entries of the next batch are requested before the neighbour records
// of the current one (position offsets and mass, one 16-byte load each, plus
// whatever extra(j) loads), and all of a batch's records are requested before
// any is used, so the list stream and the dependent gathers overlap.  Then,
// if the list overflowed, the remaining neighbours come from a re-traversal.
// fn(ok, j, rx, ry, rz, mj, x) is called for every slot of a batch (x =
// extra(j)); ok is false for the padding of the last batch (its data are
// those of a valid neighbour, its contribution must be dropped).  done() is
// called after every batch.  With a list skin, filter keeps only the
// neighbours (ok false for the others); without it a skin entry reaches fn
// with ok true -- right for terms that vanish beyond the radius (W and
// grad W of the uniform-h cubic spline are exactly 0 for q >= 2 in FP32).
template <int KX, int B, bool EXT, class Extra, class Fn, class Done>
__device__ __forceinline__ void for_listed(const Grid &g, const SrcDev &S, int cap, int64_t stride,
                                           int s, const DestPos &d, const DestDev &D, bool filter,
                                           Extra &&extra, Fn &&fn, Done &&done) {
    filter = filter && g.skin > 0.f;
    using C = Code<KX>;
    using X = decltype(extra(0));
    const int c = S.ncnt[s];
    const int m = min(c, cap);
    const uint32_t *lst = S.nbr + s;
    auto entries = [&](uint32_t (&e)[B], int k) {
        e[0] = lst[(int64_t)k * stride];
#pragma unroll
        for (int b = 1; b < B; ++b) e[b] = (k + b < m) ? lst[(int64_t)(k + b) * stride] : e[0];
    };
    uint32_t e[B];
    if (m > 0) entries(e, 0);
    const float csf = g.cs_f;
    for (int k = 0; k < m; k += B) {
        uint32_t en[B];
        const bool more = k + B < m;
        if (more) entries(en, k + B);
        float4 p[B];
        X x[B];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int j = (int)(e[b] & C::JMASK);
            p[b] = S.pm[j];
            x[b] = extra(j);
        }
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int j = (int)(e[b] & C::JMASK);
            const float3 sh = neg_cell_offset<KX>(e[b]);
            const float rx = fmaf(sh.x, csf, d.xi_x - p[b].x);
            const float ry = fmaf(sh.y, csf, d.xi_y - p[b].y);
            const float rz = fmaf(sh.z, csf, d.xi_z - p[b].z);
            fn(k + b < m && (!filter || listed_exact_test<EXT>(g, S, D, d, j, rx, ry, rz)), j, rx, ry, rz,
               p[b].w, x[b]);
        }
        done();
        if (more) {
#pragma unroll
            for (int b = 0; b < B; ++b) e[b] = en[b];
        }
    }
    if (c > cap) {
        // the list entries past cap, in the order of the list build
        int skip = cap;
        for_neighbours<KX, EXT>(g, S, d, D.x, D.y, D.z,
                           [&](int j, float rx, float ry, float rz, int, bool exact) {
                               if (skip > 0) {
                                   --skip;
                                   return;
                               }
                               if (!exact) return;
                               fn(true, j, rx, ry, rz, S.pm[j].w, extra(j));
                               done();
                           });
    }
}

// ---------------------------------------------------------------------------
// neighbour list (base/nnps.pyx:525-620 FixedDestNbrParticleLocator cache)
// ---------------------------------------------------------------------------
template <int KX, int MODE>
__global__ void __launch_bounds__(kPairBlock) k_nbrlist(const __grid_constant__ ListArgs A) {
    using C = Code<KX>;
    if (gated_off(A.gate)) return;
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int c = 0;
    if (s < A.d.n) {
        const Grid &g = grid_of<MODE == 1>(A.g, A.d, (int)s);
        DestPos d;
        if (load_dest(g, A.d, (int)s, d)) {
            uint32_t *out = A.nbr + s;
            const int cap = A.cap;
            const int64_t stride = A.stride;
            for_neighbours<KX, MODE == 2>(g, A.s, d, A.d.x, A.d.y, A.d.z,
                               [&](int j, float, float, float, int code, bool) {
                                   if (c < cap) out[(int64_t)c * stride] = (uint32_t)j | ((uint32_t)code << C::SHIFT);
                                   ++c;
                               });
        }
        A.cnt[s] = c;
    }
    const int wmax = __reduce_max_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0) atomicMax(A.maxcnt, wmax);
}

// ---------------------------------------------------------------------------
// summation density (density_funcs.pyx:38-74) + Tait (eos_funcs.pyx:105-116)
// ---------------------------------------------------------------------------
// MODE 0: one simulation; 1: a batch of simulations (per-instance grids);
// 2: one simulation with the extended search (periodic x or variable-h
// symmetric lists), kept apart so the other modes carry none of its state.
template <int KX, bool UH, int MODE>
__global__ void __launch_bounds__(kPairBlock, (UH && MODE != 2) ? 8 : 1) k_density(const __grid_constant__ DensityArgs A) {
    const int64_t s = (MODE == 1 ? A.d.s0 : 0) + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= A.d.n || gated_off(A.gate)) return;
    const Grid &g = grid_of<MODE == 1>(A.g, A.d, (int)s);
    DestPos d;
    const bool real = load_dest(g, A.d, (int)s, d);
    CSum rho;
    if (!real) {
        for (int si = 0; si < A.nsrc; ++si)
            if (A.lnbr[si] != nullptr) A.lcnt[si][s] = 0;
    }
    if (real) {
        const float hi = A.d.velh[s].w;
        const int dim = A.dim;
        const bool uh = UH;
        // a fixed h for every pair (pilot density): the variable-h kernels only
        const bool fixed = !UH && A.ih0 > 0.f;
        const float ihi = fixed ? A.ih0 : __fdividef(1.f, hi);
        const float faci = cubic_fac(dim, ihi);
        float part = 0.f;
        for (int si = 0; si < A.nsrc; ++si) {
            const SrcDev &S = A.s[si];
            if (A.lnbr[si] != nullptr) {
                // first pair pass of this build: test the stencil, write the
                // list for the passes that follow and sum in the same order
                using C = Code<KX>;
                uint32_t *out = A.lnbr[si] + s;
                const int cap = A.cap[si];
                const int64_t stride = A.stride[si];
                int c = 0;
                for_neighbours<KX, MODE == 2>(g, S, d, A.d.x, A.d.y, A.d.z,
                    [&](int j, float rx, float ry, float rz, int code, bool exact) {
                        if (c < cap) out[(int64_t)c * stride] = (uint32_t)j | ((uint32_t)code << C::SHIFT);
                        ++c;
                        if (!exact) return;
                        const float mj = S.pm[j].w;
                        float ih = ihi, fac = faci;
                        if (!uh && !fixed) {
                            ih = __fdividef(1.f, 0.5f * (hi + S.velh[j].w));
                            fac = cubic_fac(dim, ih);
                        }
                        const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                        const float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
                        rho.add(cubic_w(r * ih) * fac * mj);
                    });
                A.lcnt[si][s] = c;
                const unsigned act = __activemask();
                const int wmax = __reduce_max_sync(act, c);
                if ((threadIdx.x & 31) == (__ffs(act) - 1)) atomicMax(A.lmax[si], wmax);
                continue;
            }
            // with variable h (or a fixed h), W can reach past the radius of h_i
            for_listed<KX, (UH && MODE == 0) ? 6 : 4, MODE == 2>(g, S, A.cap[si], A.stride[si], (int)s, d, A.d, !uh, NoExtra(),
                [&](bool ok, int j, float rx, float ry, float rz, float mj, int) {
                    float ih = ihi, fac = faci;
                    if (!uh && !fixed) {
                        ih = __fdividef(1.f, 0.5f * (hi + S.velh[j].w));
                        fac = cubic_fac(dim, ih);
                    }
                    const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                    const float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
                    const float w = cubic_w(r * ih) * fac * mj;
                    part += ok ? w : 0.f;
                },
                [&]() {
                    rho.add(part);
                    part = 0.f;
                });
        }
    }
    const int orig = d.orig;
    const double r64 = real ? rho.value() : 0.0;
    if (A.rho_out) A.rho_out[orig] = r64;
    const float rf = (float)r64;
    float pf = 0.f, cf = 0.f;
    if (A.tait) {
        if (real) {
            // p = B((rho/ro)^gamma - 1), cs = co (rho/ro)^((gamma-1)/2), through
            // log1p/expm1 of the density excess so p keeps its relative accuracy
            // as rho -> ro.
            const float B = A.co * A.co * A.ro / A.gamma;
            const float lr = log1pf((float)((r64 - (double)A.ro) / (double)A.ro));
            pf = B * expm1f(A.gamma * lr);
            cf = A.co * expf(0.5f * (A.gamma - 1.f) * lr);
        }
        A.p_out[orig] = (double)pf;
        A.cs_out[orig] = (double)cf;
    }
    if (A.st_out) {
        // the whole state record from this pass and the FP64 arrays (the
        // mass from the position record): fresh whatever it held before
        const float mi = A.d.pm[s].w;
        if (A.tait) {
            A.st_out[s] = make_float4(rf, pf / (rf * rf), cf, mi);
        } else {
            const float pold = (float)ld0(A.d.p, orig);
            A.st_out[s] = make_float4(rf, pold / (rf * rf), (float)ld0(A.d.cs, orig), mi);
        }
    }
}

// ---------------------------------------------------------------------------
// rates: PGrad (pressure_funcs.pyx:40-91), Monaghan AV (viscosity_funcs.pyx:
// 41-124), XSPH (xsph_funcs.pyx:31-88), Monaghan BF (boundary_funcs.pyx:
// 54-110), gravity (external_force.pyx:39-45), stepping (position_funcs.pyx)
// ---------------------------------------------------------------------------
// velocity (+h) and state records of one neighbour
struct VelState {
    float4 v, st;
};

// SPEC 0: any terms, runtime flags; 1: PGrad + AV, uniform h, one source;
// 2: PGrad + AV + XSPH, uniform h, one source.
template <int KX, int SPEC, int MODE>
__global__ void __launch_bounds__(kPairBlock) k_rates(const __grid_constant__ RatesArgs A) {
    constexpr uint32_t SF = SPEC == 1 ? (SPH_TERM_PGRAD | SPH_TERM_AVISC)
                          : (SPEC == 2 ? (SPH_TERM_PGRAD | SPH_TERM_AVISC | SPH_TERM_XSPH) : 0u);
    constexpr bool MAY_XSPH = SPEC != 1;
    constexpr bool MAY_BF = SPEC == 0;
    constexpr bool MAY_DRHO = SPEC == 0;
    const int64_t s = (MODE == 1 ? A.d.s0 : 0) + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= A.d.n || gated_off(A.gate)) return;
    const Grid &g = grid_of<MODE == 1>(A.g, A.d, (int)s);
    DestPos d;
    const bool real = load_dest(g, A.d, (int)s, d);
    CSum ax, ay, az, xx, xy, xz, dr;
    if (real) {
        const float4 vi = A.d.velh[s];
        const float4 sti = A.d.st[s];
        const float hi = vi.w, rhoi = sti.x, pri = sti.y, ci = sti.z, mi = sti.w;
        const int dim = A.dim;
        const bool uh = SPEC != 0 || g.uniform_h != 0;
        const float ihi = __fdividef(1.f, hi);
        const float faci = cubic_fac(dim, ihi);
        float pax = 0.f, pay = 0.f, paz = 0.f, pxx = 0.f, pxy = 0.f, pxz = 0.f, pdr = 0.f;
        const int nsrc = SPEC != 0 ? 1 : A.nsrc;
        for (int si = 0; si < nsrc; ++si) {
            const SrcDev &S = A.s[si];
            const uint32_t fl = SPEC != 0 ? SF : S.flags;
            // the boundary force has its own support (normal distance, delp)
            const bool filt = !uh || (fl & SPH_TERM_BFORCE) != 0;
            for_listed<KX, (SPEC != 0 ? 3 : 2), MODE == 2>(g, S, A.cap[si], A.stride[si], (int)s, d, A.d, filt,
                [&](int j) { return VelState{S.velh[j], S.st[j]}; },
                [&](bool ok, int j, float rx, float ry, float rz, float mj, const VelState &vs) {
                const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                const float4 vj = vs.v;
                const float4 stj = vs.st;
                float hab = hi, ih = ihi, fac = faci;
                if (!uh) {
                    hab = 0.5f * (hi + vj.w);
                    ih = __fdividef(1.f, hab);
                    fac = cubic_fac(dim, ih);
                }
                const float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
                const float q = r2 * rinv * ih;
                const float okf = ok ? 1.f : 0.f;
                if (fl & (SPH_TERM_PGRAD | SPH_TERM_AVISC)) {
                    float t = 0.f;
                    if (fl & SPH_TERM_PGRAD) t = -mj * (pri + stj.y);
                    if (fl & SPH_TERM_AVISC) {
                        // Pi_ab only for approaching pairs (v_ab . r_ab < 0), as a select
                        const float dot = (vi.x - vj.x) * rx + (vi.y - vj.y) * ry + (vi.z - vj.z) * rz;
                        const bool neg = dot < 0.f;
                        const float den = neg ? fmaf(S.eta2 * hab, hab, r2) : 1.f;
                        const float mu = neg ? __fdividef(hab * dot, den) : 0.f;
                        const float cab = 0.5f * (ci + stj.z);
                        const float rhoab = 0.5f * (rhoi + stj.x);
                        const float piab = __fdividef(fmaf(S.beta * mu, mu, -S.alpha * cab * mu), rhoab);
                        t -= mj * (neg ? piab : 0.f);
                    }
                    const float gf = cubic_gfac(q, ih, rinv) * fac * t * okf;
                    pax = fmaf(gf, rx, pax);
                    pay = fmaf(gf, ry, pay);
                    paz = fmaf(gf, rz, paz);
                }
                if (MAY_DRHO && (fl & (SPH_TERM_DRHO | SPH_TERM_VDIV))) {
                    // drho_i += m_j (v_i - v_j) . grad W(hab)  (density_funcs.pyx:117-158);
                    // the velocity divergence is -sum / rho_i (adke_funcs.pyx:175-226)
                    const float dot = (vi.x - vj.x) * rx + (vi.y - vj.y) * ry + (vi.z - vj.z) * rz;
                    pdr = fmaf(cubic_gfac(q, ih, rinv) * fac * mj * okf, dot, pdr);
                }
                if (MAY_XSPH && (fl & SPH_TERM_XSPH)) {
                    const float rhoab = 0.5f * (stj.x + rhoi);
                    const float temp = __fdividef(mj * (cubic_w(q) * fac), rhoab) * S.eps * okf;
                    pxx = fmaf(temp, vj.x - vi.x, pxx);
                    pxy = fmaf(temp, vj.y - vi.y, pxy);
                    pxz = fmaf(temp, vj.z - vi.z, pxz);
                }
                if (MAY_BF && (fl & SPH_TERM_BFORCE)) {
                    const float4 nj = S.nrm[j], tj = S.tan[j];
                    const float xt = rx * tj.x + ry * tj.y + rz * tj.z;
                    const float yn = rx * nj.x + ry * nj.y + rz * nj.z;
                    const float qb = yn / hi;
                    float force = 0.f;
                    const float axt = fabsf(xt);
                    if (axt <= S.delp) {
                        const float beta = 0.02f * ci * ci / yn;
                        const float tforce = 1.f - axt / S.delp;
                        float nforce;
                        if (0.f < qb && qb <= 2.f / 3.f)
                            nforce = 2.f / 3.f;
                        else if (2.f / 3.f < qb && qb <= 1.f)
                            nforce = 2.f * qb * (1.f - 0.75f * qb);
                        else if (1.f < qb && qb <= 2.f)
                            nforce = 0.5f * (2.f - qb) * (2.f - qb);
                        else
                            nforce = 0.f;
                        force = (mj / (mi + mj)) * nforce * tforce * beta;
                    }
                    if (ok) {
                        pax += force * nj.x;
                        pay += force * nj.y;
                        paz += force * nj.z;
                    }
                }
            },
            [&]() {
                ax.add(pax); ay.add(pay); az.add(paz);
                pax = pay = paz = 0.f;
                if (MAY_DRHO) {
                    dr.add(pdr);
                    pdr = 0.f;
                }
                if (MAY_XSPH) {
                    xx.add(pxx); xy.add(pxy); xz.add(pxz);
                    pxx = pxy = pxz = 0.f;
                }
            });
        }
    }
    const int orig = d.orig;
    double a3[3] = {0.0, 0.0, 0.0}, p3[3] = {0.0, 0.0, 0.0};
    if (real) {
        a3[0] = ax.value(); a3[1] = ay.value(); a3[2] = az.value();
        p3[0] = xx.value(); p3[1] = xy.value(); p3[2] = xz.value();
        if (A.add_gravity) { a3[0] += A.gx; a3[1] += A.gy; a3[2] += A.gz; }
        if (A.add_velocity) {
            // exact FP64 velocity of the destination (position_funcs.pyx:47-50)
            p3[0] += ld0(A.d.u, orig);
            p3[1] += ld0(A.d.v, orig);
            p3[2] += ld0(A.d.w, orig);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (A.acc[c]) A.acc[c][orig] = (A.accumulate ? A.acc[c][orig] : 0.0) + a3[c];
        if (A.pos[c]) A.pos[c][orig] = (A.accumulate ? A.pos[c][orig] : 0.0) + p3[c];
    }
    if (A.drho) {
        double r = real ? dr.value() : 0.0;
        if (A.vdiv && real) r = -r / A.d.rho[orig];
        A.drho[orig] = (A.accumulate ? A.drho[orig] : 0.0) + r;
    }
}

// ---------------------------------------------------------------------------
// features of the learned momentum closure: the 32 nearest neighbours within
// the search radius (self included), ordered by squared distance then source
// slot, each as ((x_i-x_j)/h_i, (y_i-y_j)/h_i, (u_j-u_i)/c0, (v_j-v_i)/c0,
// rho_j, p_j), standardised per channel; missing neighbours are zero rows.
// Replaces the inputs of the momentum pair loop (pressure_funcs.pyx:40-91,
// viscosity_funcs.pyx:41-124) for the network.
// ---------------------------------------------------------------------------
struct FeatureArgs {
    Grid g;
    DestDev d;
    SrcDev s;
    int cap;
    int64_t stride;
    float inv_c0;
    float mean[SPH_MLP_NCH], inv_std[SPH_MLP_NCH];
    uint16_t *out_bf;   // [n][192] BF16 by original index (or null)
    float *out_f;       // [n][192] FP32 by original index (or null)
    const int *s_skey;  // sorted: cell of each source slot
    const unsigned *gate;
};

template <int KX, bool EXT>
__global__ void __launch_bounds__(kPairBlock) k_features(const __grid_constant__ FeatureArgs A) {
    constexpr int NN = SPH_MLP_NNBR, NC = SPH_MLP_NCH;
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= A.d.n || gated_off(A.gate)) return;
    DestPos d;
    const bool real = load_dest(A.g, A.d, (int)s, d);
    float kr2[NN], krx[NN], kry[NN];
    int kj[NN];
    int cnt = 0;
    if (real) {
        const SrcDev &S = A.s;
        auto keep = [&](int j, float rx, float ry, float rz) {
            const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
            if (cnt == NN && !(r2 < kr2[NN - 1] || (r2 == kr2[NN - 1] && j < kj[NN - 1]))) return;
            int k = cnt < NN ? cnt++ : NN - 1;
            while (k > 0 && (kr2[k - 1] > r2 || (kr2[k - 1] == r2 && kj[k - 1] > j))) {
                kr2[k] = kr2[k - 1]; krx[k] = krx[k - 1]; kry[k] = kry[k - 1]; kj[k] = kj[k - 1];
                --k;
            }
            kr2[k] = r2; krx[k] = rx; kry[k] = ry; kj[k] = j;
        };
        if (S.nbr) {
            const float csf = A.g.cs_f;
            using C = Code<KX>;
            const int c = S.ncnt[s];
            const int m = min(c, A.cap);
            for (int k = 0; k < m; ++k) {
                const uint32_t e = S.nbr[s + (int64_t)k * A.stride];
                const int j = (int)(e & C::JMASK);
                const float3 sh = neg_cell_offset<KX>(e);
                const float4 p = S.pm[j];
                const float rx = fmaf(sh.x, csf, d.xi_x - p.x);
                const float ry = fmaf(sh.y, csf, d.xi_y - p.y);
                const float rz = fmaf(sh.z, csf, d.xi_z - p.z);
                if (listed_exact<EXT>(A.g, S, A.d, d, j, rx, ry, rz)) keep(j, rx, ry, rz);
            }
            if (c > A.cap) {
                int skip = A.cap;
                for_neighbours<KX, EXT>(A.g, S, d, A.d.x, A.d.y, A.d.z,
                                   [&](int j, float rx, float ry, float rz, int, bool exact) {
                                       if (skip > 0) { --skip; return; }
                                       if (exact) keep(j, rx, ry, rz);
                                   });
            }
        } else {
            for_neighbours<KX, EXT>(A.g, S, d, A.d.x, A.d.y, A.d.z,
                               [&](int j, float rx, float ry, float rz, int, bool exact) {
                                   if (exact) keep(j, rx, ry, rz);
                               });
        }
    }
    const float4 vi = A.d.velh[s];
    const float ih = 1.f / vi.w;
    const int64_t row = (int64_t)d.orig * (NN * NC);
#pragma unroll 1
    for (int k = 0; k < NN; k += 4) {
        float f[4 * NC];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float raw[NC] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            const bool have = k + q < cnt;
            if (have) {
                const int j = kj[k + q];
                const float4 vj = A.s.velh[j];
                const float4 st = A.s.st[j];
                raw[0] = krx[k + q] * ih;
                raw[1] = kry[k + q] * ih;
                raw[2] = (vj.x - vi.x) * A.inv_c0;
                raw[3] = (vj.y - vi.y) * A.inv_c0;
                raw[4] = st.x;
                raw[5] = st.y * st.x * st.x;
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) f[q * NC + c] = have ? (raw[c] - A.mean[c]) * A.inv_std[c] : 0.f;
        }
        if (A.out_bf) {
            uint32_t w[12];
#pragma unroll
            for (int i = 0; i < 12; ++i) {
                __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
                w[i] = *reinterpret_cast<uint32_t *>(&h);
            }
            uint4 *o = reinterpret_cast<uint4 *>(A.out_bf + row + k * NC);
            o[0] = make_uint4(w[0], w[1], w[2], w[3]);
            o[1] = make_uint4(w[4], w[5], w[6], w[7]);
            o[2] = make_uint4(w[8], w[9], w[10], w[11]);
        }
        if (A.out_f) {
            float4 *o = reinterpret_cast<float4 *>(A.out_f + row + k * NC);
#pragma unroll
            for (int i = 0; i < 6; ++i) o[i] = make_float4(f[4 * i], f[4 * i + 1], f[4 * i + 2], f[4 * i + 3]);
        }
    }
}

// The same features with one warp per destination (no periodic axis or
// symmetry plane): lane k takes list entry k of every chunk of 32, the warp
// sorts the chunk's 64-bit keys (FP32 squared distance bits, sorted slot:
// the order of the thread-per-destination kernel) with a bitonic network
// of shuffles and merges them into the 32 nearest so far; lane k then
// recomputes the offsets of neighbour k with the list pass's operations
// (the cell offset from the source's cell) and writes row k (a
// destination's 384-byte row as one contiguous warp store).  Neighbours
// past an over-full list come from the traversal the thread-per-destination
// kernel uses, run in lockstep by all lanes (the same destination), each
// inserted into the sorted set with its own offsets.
__device__ __forceinline__ uint64_t feat_key(float r2, int j) {
    return ((uint64_t)__float_as_uint(r2) << 32) | (uint32_t)j;
}

// compare-exchange stages j0, j0/2, .., 1 of a bitonic network of block k
// (one 64-bit comparison: the partner's key is taken when it is smaller on
// a lane that keeps the minimum, larger on one that keeps the maximum;
// equal keys are alike either way)
__device__ __forceinline__ void feat_stages(uint64_t &key, int lane, int k, int j0) {
#pragma unroll
    for (int jj = j0; jj > 0; jj >>= 1) {
        const uint64_t o = __shfl_xor_sync(0xffffffffu, key, jj);
        const bool keep_max = ((lane & k) != 0) != ((lane & jj) != 0);
        if ((o < key) != keep_max) key = o;
    }
}

__device__ __forceinline__ void feat_sort32(uint64_t &key, int lane) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) feat_stages(key, lane, k, k >> 1);
}

// (six blocks per SM, 40 registers: 49 us at 80 000 destinations in 2D;
// four and eight blocks per SM measured slower)
template <int KX>
__global__ void __launch_bounds__(256, 6) k_features_warp(const __grid_constant__ FeatureArgs A) {
    constexpr int NN = SPH_MLP_NNBR, NC = SPH_MLP_NCH;
    static_assert(NN == 32, "one lane per kept neighbour");
    const int lane = threadIdx.x & 31;
    const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (s >= A.d.n || gated_off(A.gate)) return;
    DestPos d;
    const bool real = load_dest(A.g, A.d, (int)s, d);
    const SrcDev &S = A.s;
    const float csf = A.g.cs_f;
    constexpr uint64_t none = ~0ull;
    uint64_t best = none;
    // offsets carried by neighbours found by the traversal (flag set)
    float crx = 0.f, cry = 0.f;
    bool carried = false;
    if (real) {
        using C = Code<KX>;
        const int c = S.ncnt[s];
        const int m = min(c, A.cap);
        auto candidate = [&](int k) {
            uint64_t key = none;
            if (k < m) {
                const uint32_t e = S.nbr[s + (int64_t)k * A.stride];
                const int j = (int)(e & C::JMASK);
                const float3 sh = neg_cell_offset<KX>(e);
                const float4 p = S.pm[j];
                const float rx = fmaf(sh.x, csf, d.xi_x - p.x);
                const float ry = fmaf(sh.y, csf, d.xi_y - p.y);
                const float rz = fmaf(sh.z, csf, d.xi_z - p.z);
                if (listed_exact<false>(A.g, S, A.d, d, j, rx, ry, rz))
                    key = feat_key(fmaf(rx, rx, fmaf(ry, ry, rz * rz)), j);
            }
            return key;
        };
        // the 32 smallest of two ascending sets: a bitonic sequence, then merged
        auto merge = [&](uint64_t cand) {
            const uint64_t r = __shfl_sync(0xffffffffu, cand, 31 - lane);
            if (r < best) best = r;
            feat_stages(best, lane, 32, 16);
        };
        // one chunk of 32 at a time (two side by side spilled registers)
        for (int k0 = 0; k0 < m; k0 += 32) {
            uint64_t c0 = candidate(k0 + lane);
            feat_sort32(c0, lane);
            if (k0 == 0) best = c0;
            else merge(c0);
        }
        if (c > A.cap) {
            // the rest, in the order of the list build, every lane alike
            int skip = A.cap;
            for_neighbours<KX, false>(A.g, S, d, A.d.x, A.d.y, A.d.z,
                [&](int j, float rx, float ry, float rz, int, bool exact) {
                    if (skip > 0) { --skip; return; }
                    if (!exact) return;
                    const uint64_t x = feat_key(fmaf(rx, rx, fmaf(ry, ry, rz * rz)), j);
                    // insert: lanes past the position shift up by one
                    const int pos = __popc(__ballot_sync(0xffffffffu, best < x));
                    const int from = lane > 0 ? lane - 1 : 0;
                    const uint64_t pk = __shfl_sync(0xffffffffu, best, from);
                    const float px = __shfl_sync(0xffffffffu, crx, from);
                    const float py = __shfl_sync(0xffffffffu, cry, from);
                    const bool pc = __shfl_sync(0xffffffffu, carried, from);
                    if (lane > pos) {
                        best = pk; crx = px; cry = py; carried = pc;
                    } else if (lane == pos) {
                        best = x; crx = rx; cry = ry; carried = true;
                    }
                });
        }
    }
    const bool have = best != none;
    float raw[NC] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    // (loaded here, beside the neighbour's records, not live through the sort)
    const float4 vi = A.d.velh[s];
    if (have) {
        const int j = (int)(uint32_t)best;
        float rx = crx, ry = cry;
        if (!carried) {
            // the list pass's offsets: cell offset from the source's cell
            int cxj, cyj, czj;
            decode_cell(A.g, A.s_skey[j], cxj, cyj, czj);
            const float4 p = S.pm[j];
            rx = fmaf((float)(d.cx - cxj), csf, d.xi_x - p.x);
            ry = fmaf((float)(d.cy - cyj), csf, d.xi_y - p.y);
        }
        const float ih = 1.f / vi.w;
        const float4 vj = S.velh[j];
        const float4 st = S.st[j];
        raw[0] = rx * ih;
        raw[1] = ry * ih;
        raw[2] = (vj.x - vi.x) * A.inv_c0;
        raw[3] = (vj.y - vi.y) * A.inv_c0;
        raw[4] = st.x;
        raw[5] = st.y * st.x * st.x;
    }
    float f[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) f[q] = have ? (raw[q] - A.mean[q]) * A.inv_std[q] : 0.f;
    const int64_t row = (int64_t)d.orig * (NN * NC) + lane * NC;
    if (A.out_bf) {
        uint32_t *o = reinterpret_cast<uint32_t *>(A.out_bf + row);
#pragma unroll
        for (int i = 0; i < NC / 2; ++i) {
            __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
            o[i] = *reinterpret_cast<uint32_t *>(&h);
        }
    }
    if (A.out_f) {
        float2 *o = reinterpret_cast<float2 *>(A.out_f + row);
#pragma unroll
        for (int i = 0; i < NC / 2; ++i) o[i] = make_float2(f[2 * i], f[2 * i + 1]);
    }
}

DestDev make_dest(const ArraySnap &D) {
    DestDev d;
    d.pm = D.pm; d.velh = D.velh; d.st = D.st;
    d.skey = D.skey; d.perm = D.perm;
    d.sinst = nullptr; d.grids = nullptr;
    d.tag = D.view.tag;
    d.x = D.view.x; d.y = D.view.y; d.z = D.view.z;
    d.u = D.view.u; d.v = D.view.v; d.w = D.view.w;
    d.h = D.view.h;
    d.p = D.view.p;
    d.rho = D.view.rho;
    d.cs = D.view.cs;
    d.n = D.n;
    d.s0 = 0;
    return d;
}

SrcDev make_src(const ArraySnap &S) {
    SrcDev s{};
    s.velh = S.velh; s.st = S.st; s.nrm = S.nrm; s.tan = S.tan; s.pm = S.pm; s.scx = S.scx;
    s.cstart = S.cstart; s.perm = S.perm;
    s.x = S.view.x; s.y = S.view.y; s.z = S.view.z; s.h = S.view.h;
    return s;
}

int blocks_for(int64_t n) {
    return (int)std::max<int64_t>(1, (n + kPairBlock - 1) / kPairBlock);
}

// List capacity override (environment SPH_LIST_CAP, >= 1): forces the
// re-traversal path of destinations with more neighbours than the capacity.
int cap_override() {
    static int v = -2;
    if (v == -2) {
        const char *e = getenv("SPH_LIST_CAP");
        v = e ? atoi(e) : -1;
        if (v < 1) v = -1;
    }
    return v;
}

// default list capacity before the first count is known
int default_cap(const Grid &g) {
    if (g.kz > 0) return 96;
    if (g.ky > 0) return 40;
    return 16;
}

// code variant of the context's build: the stencil half-width, or 4 for
// half-width 2 with base-5 offsets
int code_variant(const sph_ctx *ctx) {
    return (ctx->grid.kx == 2 && ctx->wide_codes) ? 4 : ctx->grid.kx;
}

int64_t code_limit(int variant) {
    switch (variant) {
        case 1: return 1ll << Code<1>::SHIFT;
        case 2: return 1ll << Code<2>::SHIFT;
        case 4: return 1ll << Code<4>::SHIFT;
        default: return 1ll << Code<3>::SHIFT;
    }
}

// Allocate / size the neighbour list of (dst, src) for the current build
// (no launch).  *stale tells whether its contents must be (re)built.
// brick: the brick-staged list of the pair (16-bit staging indices), kept
// apart from the list-streaming one.
int prepare_list(sph_ctx *ctx, int dst, int src, NbrList **out, bool *stale, bool brick = false) {
    const int na = (int)ctx->arrays.size();
    if ((int)ctx->lists.size() < 2 * na * na) ctx->lists.resize((size_t)2 * na * na);
    const int slot = (brick ? na * na : 0) + dst * na + src;
    NbrList &L = ctx->lists[(size_t)slot];
    L.brick = brick;
    *out = &L;
    *stale = L.build != ctx->build_id;
    if (!*stale) return SPH_OK;
    ArraySnap &D = ctx->arrays[dst];
    ArraySnap &S = ctx->arrays[src];
    const Grid &g = ctx->grid;
    if (!brick && S.n >= code_limit(code_variant(ctx)))
        return set_error(SPH_ERR_NOTSUP, "neighbour list: too many source particles for this "
                                         "cell subdivision (use a smaller subdivision)");
    if (!L.maxcnt) {
        if (slot < kMaxListSlots) {
            L.maxcnt = (int *)(ctx->d_status + kListWord0 + slot);
        } else {
            SPH_CUDA(cudaMalloc(&L.maxcnt, sizeof(int)));
            L.own_maxcnt = true;
        }
        SPH_CUDA(cudaMemsetAsync(L.maxcnt, 0, sizeof(int), ctx->stream));
    }
    // capacity: largest count seen so far plus headroom (dests beyond it are
    // completed by re-traversal, so a short list is slow, never wrong)
    int cap = L.cap > 0 ? L.cap : default_cap(g);
    if (L.seen_max > 0) {
        const int want = (L.seen_max + L.seen_max / 4 + 15) / 8 * 8;
        if (want > cap || want < cap / 2) cap = want;
    }
    if (cap_override() > 0) cap = cap_override();
    // brick lists hold their entries in groups of 8
    if (brick) cap = (cap + 7) / 8 * 8;
    const int64_t stride = std::max<int64_t>(D.n, 1);
    const int64_t need = stride * cap;
    const bool have = brick ? L.nbr16 != nullptr : L.nbr != nullptr;
    if (need > L.entries || !have || !L.cnt || stride > L.stride_cap) {
        cudaFree(L.nbr);
        cudaFree(L.nbr16);
        cudaFree(L.cnt);
        L.nbr = nullptr;
        L.nbr16 = nullptr;
        L.cnt = nullptr;
        if (brick) SPH_CUDA(cudaMalloc(&L.nbr16, sizeof(uint16_t) * need));
        else SPH_CUDA(cudaMalloc(&L.nbr, sizeof(uint32_t) * need));
        SPH_CUDA(cudaMalloc(&L.cnt, sizeof(int) * stride));
        L.entries = need;
        L.stride_cap = stride;
    }
    L.cap = cap;
    L.stride = stride;
    return SPH_OK;
}

// Build (if stale) the neighbour list of (dst, src) for the current build.
int ensure_list(sph_ctx *ctx, int dst, int src, NbrList **out) {
    bool stale = false;
    int rc = prepare_list(ctx, dst, src, out, &stale);
    if (rc || !stale) return rc;
    if (ctx->capturing) {
        // lists are built at the positions of the build, not inside a step graph
        ctx->capture_failed = true;
        ctx->capture_fail_site = 2;   // a list to build
        return SPH_OK;
    }
    NbrList &L = **out;
    ArraySnap &D = ctx->arrays[dst];
    ArraySnap &S = ctx->arrays[src];
    const Grid &g = ctx->grid;
    if (D.n > 0) {
        ListArgs a{};
        a.g = g;
        a.d = make_dest(D);
        a.s = make_src(S);
        a.nbr = L.nbr;
        a.cnt = L.cnt;
        a.maxcnt = L.maxcnt;
        a.stride = L.stride;
        a.cap = L.cap;
        a.gate = ctx->gate;
        const int b = blocks_for(D.n);
        const bool ext = g.periodic || g.symmetric;
#define LLAUNCH(K) (ext ? k_nbrlist<K, 2><<<b, kPairBlock, 0, ctx->stream>>>(a) \
                        : k_nbrlist<K, 0><<<b, kPairBlock, 0, ctx->stream>>>(a))
        switch (code_variant(ctx)) {
            case 1: LLAUNCH(1); break;
            case 2: LLAUNCH(2); break;
            case 4: LLAUNCH(4); break;
            default: LLAUNCH(3); break;
        }
#undef LLAUNCH
        count_launch();
        SPH_LAUNCH_CHECK("k_nbrlist");
    }
    L.build = ctx->build_id;
    return SPH_OK;
}

}  // namespace

// Queue the publication of the status block (error word, displacement,
// stale flag, list maxima) to its mapped host mirror, read after the next
// synchronisation.
int list_maxima_async(sph_ctx *ctx) {
    const int nl = std::min((int)ctx->lists.size(), kMaxListSlots);
    return publish_words(ctx, ctx->d_status, ctx->hd_status, kListWord0 + nl);
}

void list_maxima_collect(sph_ctx *ctx) {
    const int nl = (int)ctx->lists.size();
    for (int i = 0; i < nl && i < kMaxListSlots; ++i)
        if (ctx->lists[i].maxcnt)
            ctx->lists[i].seen_max = std::max(ctx->lists[i].seen_max, (int)ctx->h_status[kListWord0 + i]);
}

void free_lists(sph_ctx *ctx) {
    for (auto &L : ctx->lists) {
        cudaFree(L.nbr);
        cudaFree(L.nbr16);
        cudaFree(L.cnt);
        if (L.own_maxcnt) cudaFree(L.maxcnt);
    }
    ctx->lists.clear();
}

int build_lists(sph_ctx *ctx, int dst, const int *srcs, int nsrc) {
    if (!ctx->built) return set_error(SPH_ERR_STATE, "lists: no neighbour build");
    const int na = (int)ctx->arrays.size();
    if (dst < 0 || dst >= na || nsrc < 0 || (nsrc > 0 && !srcs))
        return set_error(SPH_ERR_ARG, "lists: bad destination / sources");
    for (int i = 0; i < nsrc; ++i) {
        if (srcs[i] < 0 || srcs[i] >= na) return set_error(SPH_ERR_ARG, "lists: bad source");
        NbrList *L;
        const int rc = ensure_list(ctx, dst, srcs[i], &L);
        if (rc) return rc;
    }
    return SPH_OK;
}

namespace {

// A pair pass after a deferred light refresh: launched gated, then the
// refresh's status is read; if the lists were stale the gated launch did
// nothing and the pass runs again on the full build that replaced them.
template <class Pass>
int gated_pass(sph_ctx *ctx, Pass &&pass) {
    if (!ctx->pending) return pass();
    ctx->gate = ctx->d_status + kStaleWord;
    const int rc = pass();
    ctx->gate = nullptr;
    bool rebuilt = false;
    const int rr = resolve_pending(ctx, &rebuilt);
    if (rr) return rr;
    if (rc) return rc;
    return rebuilt ? pass() : SPH_OK;
}

// cs / rho^3 of the state records a density pass with these parameters
// writes, when its Tait equation has gamma = 7 (0 otherwise)
static double st_tait_factor(const sph_density_params *prm) {
    if (!prm->tait || prm->gamma != 7.0 || !(prm->ro > 0.0)) return 0.0;
    return prm->co / (prm->ro * prm->ro * prm->ro);
}

int density_pass(sph_ctx *ctx, int dst, const int *srcs, int nsrc, const sph_density_params *prm,
                 double *rho, double *p, double *cs) {
    if (!ctx->built) return set_error(SPH_ERR_STATE, "density: no neighbour build");
    const int na = (int)ctx->arrays.size();
    if (dst < 0 || dst >= na || nsrc < 0 || nsrc > SPH_MAX_SOURCES || !prm)
        return set_error(SPH_ERR_ARG, "density: bad destination / sources");
    ArraySnap &D = ctx->arrays[dst];
    if (prm->h0 < 0.0) return set_error(SPH_ERR_ARG, "density: h0 must be >= 0");
    for (int i = 0; i < nsrc; ++i)
        if (srcs[i] < 0 || srcs[i] >= na) return set_error(SPH_ERR_ARG, "density: bad source");
    if (brick_density_eligible(ctx, dst, srcs, nsrc, prm)) {
        NbrList *L;
        bool stale = false;
        const int rc = prepare_list(ctx, dst, srcs[0], &L, &stale, true);
        if (rc) return rc;
        if (stale && ctx->capturing) {
            ctx->capture_failed = true;
            ctx->capture_fail_site = 3;   // a list to build
            return SPH_OK;
        }
        const bool own = rho != nullptr && rho == D.view.rho &&
                         (!prm->tait || (p == D.view.p && cs == D.view.cs));
        const int rb = brick_density(ctx, dst, srcs[0], *L, stale, true, prm, rho, p, cs,
                                     own ? D.st : nullptr);
        if (rb) return rb;
        if (own) {
            D.st_fresh = true;
            D.st_tait_f = st_tait_factor(prm);
        }
        if (stale) L->build = ctx->build_id;
        ctx->n_brick_passes += 1;
        return SPH_OK;
    }
    DensityArgs a{};
    a.g = ctx->grid;
    a.d = make_dest(D);
    a.nsrc = nsrc;
    NbrList *built[SPH_MAX_SOURCES] = {nullptr};
    for (int i = 0; i < nsrc; ++i) {
        if (srcs[i] < 0 || srcs[i] >= na) return set_error(SPH_ERR_ARG, "density: bad source");
        for (int k = 0; k < i; ++k)
            if (srcs[k] == srcs[i]) return set_error(SPH_ERR_ARG, "density: repeated source");
        NbrList *L;
        bool stale = false;
        const int rc = prepare_list(ctx, dst, srcs[i], &L, &stale);
        if (rc) return rc;
        if (stale && ctx->capturing) {
            ctx->capture_failed = true;
            ctx->capture_fail_site = 4;   // a list to build
            return SPH_OK;
        }
        a.s[i] = make_src(ctx->arrays[srcs[i]]);
        a.s[i].nbr = L->nbr;
        a.s[i].ncnt = L->cnt;
        a.cap[i] = L->cap;
        a.stride[i] = L->stride;
        if (stale) {
            a.lnbr[i] = L->nbr;
            a.lcnt[i] = L->cnt;
            a.lmax[i] = L->maxcnt;
            built[i] = L;
        }
    }
    a.dim = prm->dim;
    a.tait = prm->tait;
    a.co = (float)prm->co; a.ro = (float)prm->ro; a.gamma = (float)prm->gamma;
    a.rho_out = rho; a.p_out = p; a.cs_out = cs;
    // the sorted state of the destination follows its own rho (and p, cs with
    // Tait); a density written to some other property leaves it untouched
    const bool own = rho != nullptr && rho == D.view.rho &&
                     (!prm->tait || (p == D.view.p && cs == D.view.cs));
    a.st_out = own ? D.st : nullptr;
    a.gate = ctx->gate;
    if (prm->h0 < 0.0) return set_error(SPH_ERR_ARG, "density: h0 must be >= 0");
    a.ih0 = prm->h0 > 0.0 ? (float)(1.0 / prm->h0) : 0.f;
    if (D.n == 0) return SPH_OK;
    const int b = blocks_for(D.n);
    // a fixed h (pilot density) runs in the variable-h kernels
    const bool uh = a.g.uniform_h != 0 && a.ih0 == 0.f;
    const bool ext = a.g.periodic || a.g.symmetric;
#define DLAUNCH(K) (ext ? (uh ? k_density<K, true, 2><<<b, kPairBlock, 0, ctx->stream>>>(a) \
                              : k_density<K, false, 2><<<b, kPairBlock, 0, ctx->stream>>>(a)) \
                        : (uh ? k_density<K, true, 0><<<b, kPairBlock, 0, ctx->stream>>>(a) \
                              : k_density<K, false, 0><<<b, kPairBlock, 0, ctx->stream>>>(a)))
    switch (code_variant(ctx)) {
        case 1: DLAUNCH(1); break;
        case 2: DLAUNCH(2); break;
        case 4: DLAUNCH(4); break;
        default: DLAUNCH(3); break;
    }
#undef DLAUNCH
    count_launch();
    SPH_LAUNCH_CHECK("k_density");
    if (a.st_out) {
        D.st_fresh = true;   // every slot's state record rewritten
        D.st_tait_f = st_tait_factor(prm);
    }
    for (int i = 0; i < nsrc; ++i)
        if (built[i]) built[i]->build = ctx->build_id;
    return SPH_OK;
}

int rates_pass(sph_ctx *ctx, int dst, const sph_source_term *terms, int nterms,
               const sph_rates_params *prm, double *const *acc, double *const *pos,
               int accumulate) {
    if (!ctx->built) return set_error(SPH_ERR_STATE, "rates: no neighbour build");
    const int na = (int)ctx->arrays.size();
    if (dst < 0 || dst >= na || nterms < 0 || nterms > SPH_MAX_SOURCES || !prm)
        return set_error(SPH_ERR_ARG, "rates: bad destination / sources");
    ArraySnap &D = ctx->arrays[dst];
    {
        int rc = ensure_state(ctx, dst);
        for (int i = 0; !rc && i < nterms; ++i)
            if (terms[i].src >= 0 && terms[i].src < na) rc = ensure_state(ctx, terms[i].src);
        if (rc) return rc;
    }
    for (int i = 0; i < nterms; ++i)
        if (terms[i].src < 0 || terms[i].src >= na) return set_error(SPH_ERR_ARG, "rates: bad source");
    if (brick_rates_eligible(ctx, dst, terms, nterms, prm)) {
        NbrList *L;
        bool stale = false;
        int rc = prepare_list(ctx, dst, terms[0].src, &L, &stale, true);
        if (rc) return rc;
        if (stale && ctx->capturing) {
            ctx->capture_failed = true;
            ctx->capture_fail_site = 5;   // a list to build
            return SPH_OK;
        }
        if (stale) {
            // no density pass of this build wrote the list: build it alone
            rc = brick_density(ctx, dst, terms[0].src, *L, true, false, nullptr, nullptr, nullptr,
                               nullptr, nullptr);
            if (rc) return rc;
            L->build = ctx->build_id;
        }
        rc = brick_rates(ctx, dst, terms[0], *L, prm, acc, pos, accumulate);
        if (rc) return rc;
        ctx->n_brick_passes += 1;
        return SPH_OK;
    }
    RatesArgs a{};
    a.g = ctx->grid;
    a.d = make_dest(D);
    a.nsrc = nterms;
    for (int i = 0; i < nterms; ++i) {
        const int s = terms[i].src;
        if (s < 0 || s >= na) return set_error(SPH_ERR_ARG, "rates: bad source");
        if ((terms[i].flags & SPH_TERM_BFORCE) && !ctx->arrays[s].has_nrm)
            return set_error(SPH_ERR_ARG, "rates: boundary force source has no normals");
        NbrList *L;
        const int rc = ensure_list(ctx, dst, s, &L);
        if (rc) return rc;
        a.s[i] = make_src(ctx->arrays[s]);
        a.s[i].nbr = L->nbr;
        a.s[i].ncnt = L->cnt;
        a.cap[i] = L->cap;
        a.stride[i] = L->stride;
        a.s[i].flags = terms[i].flags;
        a.s[i].alpha = (float)terms[i].alpha;
        a.s[i].beta = (float)terms[i].beta;
        a.s[i].eta2 = (float)(terms[i].eta * terms[i].eta);
        a.s[i].eps = (float)terms[i].eps;
        a.s[i].delp = (float)terms[i].delp;
    }
    a.dim = prm->dim;
    a.add_velocity = prm->add_velocity;
    a.add_gravity = prm->add_gravity;
    a.gx = prm->gx; a.gy = prm->gy; a.gz = prm->gz;
    a.accumulate = accumulate;
    for (int c = 0; c < 3; ++c) {
        a.acc[c] = acc ? acc[c] : nullptr;
        a.pos[c] = pos ? pos[c] : nullptr;
    }
    a.drho = prm->drho_out;
    a.gate = ctx->gate;
    {
        bool drho = false, vdiv = false;
        for (int i = 0; i < nterms; ++i) {
            drho = drho || (terms[i].flags & SPH_TERM_DRHO);
            vdiv = vdiv || (terms[i].flags & SPH_TERM_VDIV);
        }
        if (drho && vdiv)
            return set_error(SPH_ERR_ARG, "rates: density rate and velocity divergence in one launch");
        if (vdiv && !D.view.rho)
            return set_error(SPH_ERR_ARG, "rates: velocity divergence needs the destination's rho");
        a.vdiv = vdiv ? 1 : 0;
    }
    if (D.n == 0) return SPH_OK;
    const int b = blocks_for(D.n);
    int spec = 0;
    if (nterms == 1 && a.g.uniform_h) {
        if (terms[0].flags == (SPH_TERM_PGRAD | SPH_TERM_AVISC)) spec = 1;
        else if (terms[0].flags == (SPH_TERM_PGRAD | SPH_TERM_AVISC | SPH_TERM_XSPH)) spec = 2;
    }
    // the extended search (periodic x, variable-h lists) has its own
    // instantiation of the general kernel; the specialised ones need neither
    if (a.g.periodic || a.g.symmetric) spec = 3;
#define RLAUNCH(K) (spec == 1 ? k_rates<K, 1, 0><<<b, kPairBlock, 0, ctx->stream>>>(a) \
                    : spec == 2 ? k_rates<K, 2, 0><<<b, kPairBlock, 0, ctx->stream>>>(a) \
                    : spec == 3 ? k_rates<K, 0, 2><<<b, kPairBlock, 0, ctx->stream>>>(a) \
                                : k_rates<K, 0, 0><<<b, kPairBlock, 0, ctx->stream>>>(a))
    switch (code_variant(ctx)) {
        case 1: RLAUNCH(1); break;
        case 2: RLAUNCH(2); break;
        case 4: RLAUNCH(4); break;
        default: RLAUNCH(3); break;
    }
#undef RLAUNCH
    count_launch();
    SPH_LAUNCH_CHECK("k_rates");
    return SPH_OK;
}

int features_pass(sph_ctx *ctx, int dst, int src, const sph_mlp_feature_params *prm,
                  uint16_t *out_bf, float *out_f) {
    if (!ctx->built) return set_error(SPH_ERR_STATE, "features: no neighbour build");
    const int na = (int)ctx->arrays.size();
    if (dst < 0 || dst >= na || src < 0 || src >= na || !prm || (!out_bf && !out_f))
        return set_error(SPH_ERR_ARG, "features: bad arguments");
    if (((uintptr_t)out_bf & 15u) || ((uintptr_t)out_f & 15u))
        return set_error(SPH_ERR_ARG, "features: outputs must be 16-byte aligned");
    if (prm->c0 <= 0.0) return set_error(SPH_ERR_ARG, "features: c0 must be positive");
    ArraySnap &D = ctx->arrays[dst];
    NbrList *L;
    int rc = ensure_state(ctx, src);
    if (!rc) rc = ensure_list(ctx, dst, src, &L);
    if (rc) return rc;
    FeatureArgs a{};
    a.g = ctx->grid;
    a.d = make_dest(D);
    a.s = make_src(ctx->arrays[src]);
    a.s.nbr = L->nbr;
    a.s.ncnt = L->cnt;
    a.cap = L->cap;
    a.stride = L->stride;
    a.inv_c0 = (float)(1.0 / prm->c0);
    for (int c = 0; c < SPH_MLP_NCH; ++c) {
        a.mean[c] = prm->mean[c];
        a.inv_std[c] = prm->inv_std[c];
    }
    a.out_bf = out_bf;
    a.out_f = out_f;
    a.s_skey = ctx->arrays[src].skey;
    a.gate = ctx->gate;
    if (D.n == 0) return SPH_OK;
    const int b = blocks_for(D.n);
    const bool ext = a.g.periodic || a.g.symmetric;
    // one warp per destination (environment SPH_FEATURES_THREAD=1, read at
    // every call: one thread per destination)
    const char *env_thread = getenv("SPH_FEATURES_THREAD");
    const bool per_thread = env_thread && atoi(env_thread) > 0;
    const int bw = (int)((D.n * 32 + 255) / 256);
#define FLAUNCH(K) (ext ? k_features<K, true><<<b, kPairBlock, 0, ctx->stream>>>(a) \
                    : per_thread ? k_features<K, false><<<b, kPairBlock, 0, ctx->stream>>>(a) \
                                 : k_features_warp<K><<<bw, 256, 0, ctx->stream>>>(a))
    switch (code_variant(ctx)) {
        case 1: FLAUNCH(1); break;
        case 2: FLAUNCH(2); break;
        case 4: FLAUNCH(4); break;
        default: FLAUNCH(3); break;
    }
#undef FLAUNCH
    count_launch();
    SPH_LAUNCH_CHECK("k_features");
    return SPH_OK;
}

}  // namespace

int launch_density(sph_ctx *ctx, int dst, const int *srcs, int nsrc, const sph_density_params *prm,
                   double *rho, double *p, double *cs) {
    return gated_pass(ctx, [&] { return density_pass(ctx, dst, srcs, nsrc, prm, rho, p, cs); });
}

int launch_rates(sph_ctx *ctx, int dst, const sph_source_term *terms, int nterms,
                 const sph_rates_params *prm, double *const *acc, double *const *pos,
                 int accumulate) {
    return gated_pass(ctx, [&] {
        return rates_pass(ctx, dst, terms, nterms, prm, acc, pos, accumulate);
    });
}

int launch_features(sph_ctx *ctx, int dst, int src, const sph_mlp_feature_params *prm,
                    uint16_t *out_bf, float *out_f) {
    return gated_pass(ctx, [&] { return features_pass(ctx, dst, src, prm, out_bf, out_f); });
}

}  // namespace sphgb

// ---------------------------------------------------------------------------
// batches: the same kernels over all instances, grid per instance
// ---------------------------------------------------------------------------
namespace sphgb {

int batch_density(sph_batch *b) {
    const sph_batch_recipe &r = b->rec;
    DensityArgs a{};
    a.g = b->h_grids[0];
    a.d = make_dest(b->snap);
    a.d.sinst = b->sinst;
    a.d.grids = b->d_grids;
    a.nsrc = 1;
    a.s[0] = make_src(b->snap);
    a.s[0].nbr = b->list.nbr;
    a.s[0].ncnt = b->list.cnt;
    a.cap[0] = b->list.cap;
    a.stride[0] = b->list.stride;
    // every evaluation follows a neighbour build: the density pass writes the lists
    a.lnbr[0] = b->list.nbr;
    a.lcnt[0] = b->list.cnt;
    a.lmax[0] = b->list.maxcnt;
    a.dim = r.density.dim;
    a.tait = r.density.tait;
    a.co = (float)r.density.co; a.ro = (float)r.density.ro; a.gamma = (float)r.density.gamma;
    a.rho_out = const_cast<double *>(b->view.rho);
    a.p_out = const_cast<double *>(b->view.p);
    a.cs_out = const_cast<double *>(b->view.cs);
    a.st_out = b->snap.st;
    a.gate = b->d_err;
    const bool uh = b->uniform_h != 0;
    // one launch per group of instances of equal subdivision (their sorted
    // slots are contiguous)
    for (const BatchGroup &grp : b->groups) {
        a.d.s0 = grp.s0;
        a.d.n = grp.s1;
        const int blocks = blocks_for(grp.s1 - grp.s0);
#define BDL(K_) (uh ? k_density<K_, true, 1><<<blocks, kPairBlock, 0, b->stream>>>(a) \
                    : k_density<K_, false, 1><<<blocks, kPairBlock, 0, b->stream>>>(a))
        if (grp.K == 1) BDL(1);
        else if (grp.K == 2) BDL(2);
        else BDL(3);
#undef BDL
        count_launch();
        SPH_LAUNCH_CHECK("k_density (batch)");
    }
    return SPH_OK;
}

int batch_rates(sph_batch *b, double *const *acc, double *const *pos) {
    const sph_batch_recipe &r = b->rec;
    RatesArgs a{};
    a.g = b->h_grids[0];
    a.d = make_dest(b->snap);
    a.d.sinst = b->sinst;
    a.d.grids = b->d_grids;
    a.nsrc = 1;
    a.s[0] = make_src(b->snap);
    a.s[0].nbr = b->list.nbr;
    a.s[0].ncnt = b->list.cnt;
    a.cap[0] = b->list.cap;
    a.stride[0] = b->list.stride;
    a.s[0].flags = r.term.flags;
    a.s[0].alpha = (float)r.term.alpha;
    a.s[0].beta = (float)r.term.beta;
    a.s[0].eta2 = (float)(r.term.eta * r.term.eta);
    a.s[0].eps = (float)r.term.eps;
    a.s[0].delp = (float)r.term.delp;
    if ((r.term.flags & SPH_TERM_BFORCE))
        return set_error(SPH_ERR_NOTSUP, "batch: boundary force needs a wall array");
    a.dim = r.rates.dim;
    a.add_velocity = r.rates.add_velocity;
    a.add_gravity = r.rates.add_gravity;
    a.gx = r.rates.gx; a.gy = r.rates.gy; a.gz = r.rates.gz;
    a.accumulate = 0;
    for (int c = 0; c < 3; ++c) {
        a.acc[c] = acc[c];
        a.pos[c] = pos[c];
    }
    a.gate = b->d_err;
    int spec = 0;
    if (b->uniform_h) {
        if (r.term.flags == (SPH_TERM_PGRAD | SPH_TERM_AVISC)) spec = 1;
        else if (r.term.flags == (SPH_TERM_PGRAD | SPH_TERM_AVISC | SPH_TERM_XSPH)) spec = 2;
    }
    for (const BatchGroup &grp : b->groups) {
        a.d.s0 = grp.s0;
        a.d.n = grp.s1;
        const int blocks = blocks_for(grp.s1 - grp.s0);
#define BRL(K_) (spec == 1 ? k_rates<K_, 1, 1><<<blocks, kPairBlock, 0, b->stream>>>(a) \
                 : spec == 2 ? k_rates<K_, 2, 1><<<blocks, kPairBlock, 0, b->stream>>>(a) \
                             : k_rates<K_, 0, 1><<<blocks, kPairBlock, 0, b->stream>>>(a))
        if (grp.K == 1) BRL(1);
        else if (grp.K == 2) BRL(2);
        else BRL(3);
#undef BRL
        count_launch();
        SPH_LAUNCH_CHECK("k_rates (batch)");
    }
    return SPH_OK;
}

}  // namespace sphgb
