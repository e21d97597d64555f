// Pair-loop kernels (sm_103a): summation density (+ Tait) and the rates
// kernel (pressure gradient, Monaghan artificial viscosity, XSPH, Monaghan
// boundary force, with gravity / position stepping folded into the store).
//
// Replaces SPHCalc.sph -> SPHFunction.eval -> eval_single -> eval_nbr of the
// reference (sph/sph_calc.pyx:223-270, sph/sph_func.pyx:199-234,381-394,
// 466-484) for the functions listed in the header.  One group of LPD lanes
// owns one destination (in cell-sorted order); the stencil candidates are
// tested by all lanes, hits are queued and evaluated LPD at a time, and the
// per-lane compensated FP32 sums are combined by an error-free butterfly.
#include <cuda_runtime.h>

#include <algorithm>

#include "sph_internal.cuh"

namespace sphgb {

namespace {

struct DestDev {
    const float4 *posm, *velh, *st;
    const int *skey, *perm;
    const int64_t *tag;
    const double *x, *y, *z, *u, *v, *w, *h, *m, *cs, *rho, *p;
    int64_t n;
};

struct DensityArgs {
    Grid g;
    DestDev d;
    SrcDev s[SPH_MAX_SOURCES];
    int nsrc;
    int dim;
    int tait;
    float co, ro, gamma;
    double *rho_out, *p_out, *cs_out;
    float4 *st_out; // sorted state of the destination (may be null)
};

struct RatesArgs {
    Grid g;
    DestDev d;
    SrcDev s[SPH_MAX_SOURCES];
    int nsrc;
    int dim;
    int add_velocity, add_gravity, accumulate;
    double gx, gy, gz;
    double *acc[3];
    double *pos[3];
};

// Fill the group's destination context (identical in every lane of it).
__device__ __forceinline__ void load_dest(const Grid &g, const DestDev &D, int ds, bool valid,
                                          DestCtx &dc, int &orig, bool &real) {
    dc.active = false;
    orig = 0;
    real = false;
    dc.xi_x = dc.xi_y = dc.xi_z = 0.f;
    dc.cx = dc.cy = dc.cz = 0;
    dc.r2lo = dc.r2hi = -1.f;
    dc.px = dc.py = dc.pz = 0.0;
    dc.radius2 = -1.0;
    if (!valid) return;
    orig = D.perm[ds];
    real = (D.tag == nullptr) || (D.tag[orig] == SPH_TAG_LOCAL_REAL);
    if (!real) return;
    float4 p = D.posm[ds];
    dc.xi_x = p.x; dc.xi_y = p.y; dc.xi_z = p.z;
    decode_cell(g, D.skey[ds], dc.cx, dc.cy, dc.cz);
    double radius = __dmul_rn(D.h[orig], g.radius_scale);
    dc.radius2 = __dmul_rn(radius, radius);
    float r2 = (float)dc.radius2;
    dc.r2lo = r2 * (1.f - 1e-5f);
    dc.r2hi = r2 * (1.f + 1e-5f);
    dc.px = ld0(D.x, orig); dc.py = ld0(D.y, orig); dc.pz = ld0(D.z, orig);
    dc.active = true;
}

// ---------------------------------------------------------------------------
// summation density (density_funcs.pyx:38-74) + Tait (eos_funcs.pyx:105-116)
// ---------------------------------------------------------------------------
template <int KX, int LPD>
__global__ void __launch_bounds__(kPairBlock) k_density(const __grid_constant__ DensityArgs A) {
    __shared__ int s_qj[kPairBlock / 32][kQueue];
    __shared__ QEntry s_qe[kPairBlock / 32][kQueue];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    constexpr int G = 32 / LPD;
    const int grp = lane / LPD, gl = lane % LPD;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w0 = blockIdx.x * (int64_t)(blockDim.x >> 5) + warp; w0 * G < A.d.n; w0 += nwarps) {
        int64_t ds = w0 * G + grp;
        bool valid = ds < A.d.n;
        DestCtx dc;
        int orig;
        bool real;
        load_dest(A.g, A.d, (int)ds, valid, dc, orig, real);
        float hi = valid ? A.d.velh[ds].w : 1.f;
        CSum rho;
        const int dim = A.dim;
        for (int si = 0; si < A.nsrc; ++si) {
            const SrcDev &S = A.s[si];
            auto proc = [&](int j, const QEntry &e) {
                float hj = S.velh[j].w;
                float hab = 0.5f * (hi + hj);
                float ih = __fdividef(1.f, hab);
                float r2 = fmaf(e.r.x, e.r.x, fmaf(e.r.y, e.r.y, e.r.z * e.r.z));
                float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
                float w = cubic_w(r * ih) * cubic_fac(dim, ih);
                rho.add(w * e.r.w);
            };
            traverse<KX, LPD>(A.g, S, dc, s_qj[warp], s_qe[warp], proc);
        }
        group_reduce<LPD>(rho);
        if (valid && gl == 0) {
            double r64 = real ? rho.value() : 0.0;
            if (A.rho_out) A.rho_out[orig] = r64;
            float rf = (float)r64;
            float pf = 0.f, cf = 0.f;
            if (A.tait && real) {
                // p = B((rho/ro)^gamma - 1), cs = co (rho/ro)^((gamma-1)/2), evaluated
                // through log1p/expm1 of the density excess so that p keeps its
                // relative accuracy as rho -> ro.
                float B = A.co * A.co * A.ro / A.gamma;
                float lr = log1pf((rf - A.ro) / A.ro);
                pf = B * expm1f(A.gamma * lr);
                cf = A.co * expf(0.5f * (A.gamma - 1.f) * lr);
                if (A.p_out) A.p_out[orig] = (double)pf;
                if (A.cs_out) A.cs_out[orig] = (double)cf;
            } else if (A.tait) {
                if (A.p_out) A.p_out[orig] = 0.0;
                if (A.cs_out) A.cs_out[orig] = 0.0;
            }
            if (A.st_out) {
                float4 old = A.st_out[ds];
                if (A.tait) {
                    A.st_out[ds] = make_float4(rf, pf / (rf * rf), cf, pf);
                } else {
                    A.st_out[ds] = make_float4(rf, old.w / (rf * rf), old.z, old.w);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// rates: PGrad (pressure_funcs.pyx:40-91), Monaghan AV (viscosity_funcs.pyx:
// 41-124), XSPH (xsph_funcs.pyx:31-88), Monaghan BF (boundary_funcs.pyx:
// 54-110), gravity (external_force.pyx:39-45), stepping (position_funcs.pyx)
// ---------------------------------------------------------------------------
template <int KX, int LPD>
__global__ void __launch_bounds__(kPairBlock) k_rates(const __grid_constant__ RatesArgs A) {
    __shared__ int s_qj[kPairBlock / 32][kQueue];
    __shared__ QEntry s_qe[kPairBlock / 32][kQueue];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    constexpr int G = 32 / LPD;
    const int grp = lane / LPD, gl = lane % LPD;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w0 = blockIdx.x * (int64_t)(blockDim.x >> 5) + warp; w0 * G < A.d.n; w0 += nwarps) {
        int64_t ds = w0 * G + grp;
        bool valid = ds < A.d.n;
        DestCtx dc;
        int orig;
        bool real;
        load_dest(A.g, A.d, (int)ds, valid, dc, orig, real);
        float4 vi = valid ? A.d.velh[ds] : make_float4(0.f, 0.f, 0.f, 1.f);
        float4 sti = valid ? A.d.st[ds] : make_float4(1.f, 0.f, 0.f, 0.f);
        float mi = valid ? A.d.posm[ds].w : 0.f;
        const float hi = vi.w, rhoi = sti.x, pri = sti.y, ci = sti.z;
        CSum ax, ay, az, xx, xy, xz;
        const int dim = A.dim;
        for (int si = 0; si < A.nsrc; ++si) {
            const SrcDev &S = A.s[si];
            const uint32_t fl = S.flags;
            auto proc = [&](int j, const QEntry &e) {
                const float rx = e.r.x, ry = e.r.y, rz = e.r.z, mj = e.r.w;
                float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                float4 vj = S.velh[j];
                float hab = 0.5f * (hi + vj.w);
                float ih = __fdividef(1.f, hab);
                float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
                float q = r2 * rinv * ih;
                float fac = cubic_fac(dim, ih);
                if (fl & (SPH_TERM_PGRAD | SPH_TERM_AVISC)) {
                    float4 stj = S.st[j];
                    float t = 0.f;
                    if (fl & SPH_TERM_PGRAD) t -= mj * (pri + stj.y);
                    if (fl & SPH_TERM_AVISC) {
                        float dot = (vi.x - vj.x) * rx + (vi.y - vj.y) * ry + (vi.z - vj.z) * rz;
                        if (dot < 0.f) {
                            float cab = 0.5f * (ci + stj.z);
                            float rhoab = 0.5f * (rhoi + stj.x);
                            float mu = hab * dot / (r2 + S.eta2 * hab * hab);
                            float piab = (-S.alpha * cab * mu + S.beta * mu * mu) / rhoab;
                            t -= mj * piab;
                        }
                    }
                    float gf = cubic_gfac(q, ih, rinv) * fac * t;
                    ax.add(gf * rx);
                    ay.add(gf * ry);
                    az.add(gf * rz);
                }
                if (fl & SPH_TERM_XSPH) {
                    float rhoj = S.st[j].x;
                    float rhoab = 0.5f * (rhoj + rhoi);
                    float temp = mj * (cubic_w(q) * fac) / rhoab * S.eps;
                    xx.add(temp * (vj.x - vi.x));
                    xy.add(temp * (vj.y - vi.y));
                    xz.add(temp * (vj.z - vi.z));
                }
                if (fl & SPH_TERM_BFORCE) {
                    float4 nj = S.nrm[j], tj = S.tan[j];
                    float xt = rx * tj.x + ry * tj.y + rz * tj.z;
                    float yn = rx * nj.x + ry * nj.y + rz * nj.z;
                    float qb = yn / hi;
                    float force = 0.f;
                    float axt = fabsf(xt);
                    if (axt <= S.delp) {
                        float beta = 0.02f * ci * ci / yn;
                        float tforce = 1.f - axt / S.delp;
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
                    ax.add(force * nj.x);
                    ay.add(force * nj.y);
                    az.add(force * nj.z);
                }
            };
            traverse<KX, LPD>(A.g, S, dc, s_qj[warp], s_qe[warp], proc);
        }
        group_reduce<LPD>(ax);
        group_reduce<LPD>(ay);
        group_reduce<LPD>(az);
        group_reduce<LPD>(xx);
        group_reduce<LPD>(xy);
        group_reduce<LPD>(xz);
        if (valid && gl == 0) {
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
        }
    }
}

template <int KX, int LPD>
void launch_density_t(const DensityArgs &a, int blocks, cudaStream_t st) {
    k_density<KX, LPD><<<blocks, kPairBlock, 0, st>>>(a);
}

template <int KX, int LPD>
void launch_rates_t(const RatesArgs &a, int blocks, cudaStream_t st) {
    k_rates<KX, LPD><<<blocks, kPairBlock, 0, st>>>(a);
}

// lanes per destination: enough lanes for the expected candidate count
int choose_lpd(const Grid &g) {
    int rows = (2 * g.ky + 1) * (2 * g.kz + 1);
    if (rows >= 9) return 32;
    if (rows >= 3) return 16;
    return 8;
}

DestDev make_dest(const ArraySnap &D) {
    DestDev d;
    d.posm = D.posm; d.velh = D.velh; d.st = D.st;
    d.skey = D.skey; d.perm = D.perm;
    d.tag = D.view.tag;
    d.x = D.view.x; d.y = D.view.y; d.z = D.view.z;
    d.u = D.view.u; d.v = D.view.v; d.w = D.view.w;
    d.h = D.view.h; d.m = D.view.m; d.cs = D.view.cs;
    d.rho = D.view.rho; d.p = D.view.p;
    d.n = D.n;
    return d;
}

SrcDev make_src(const ArraySnap &S) {
    SrcDev s{};
    s.posm = S.posm; s.velh = S.velh; s.st = S.st; s.nrm = S.nrm; s.tan = S.tan;
    s.cstart = S.cstart; s.perm = S.perm;
    s.x = S.view.x; s.y = S.view.y; s.z = S.view.z;
    return s;
}

int blocks_for(int64_t n, int lpd) {
    int64_t warps = (n * lpd + 31) / 32;
    int64_t blocks = (warps + (kPairBlock / 32) - 1) / (kPairBlock / 32);
    return (int)std::max<int64_t>(1, std::min<int64_t>(blocks, 1 << 30));
}

}  // namespace

int launch_density(sph_ctx *ctx, int dst, const int *srcs, int nsrc, const sph_density_params *prm,
                   double *rho, double *p, double *cs) {
    if (!ctx->built) return set_error(SPH_ERR_STATE, "density: no neighbour build");
    int na = (int)ctx->arrays.size();
    if (dst < 0 || dst >= na || nsrc < 0 || nsrc > SPH_MAX_SOURCES || !prm)
        return set_error(SPH_ERR_ARG, "density: bad destination / sources");
    ArraySnap &D = ctx->arrays[dst];
    DensityArgs a{};
    a.g = ctx->grid;
    a.d = make_dest(D);
    a.nsrc = nsrc;
    for (int i = 0; i < nsrc; ++i) {
        if (srcs[i] < 0 || srcs[i] >= na) return set_error(SPH_ERR_ARG, "density: bad source");
        a.s[i] = make_src(ctx->arrays[srcs[i]]);
    }
    a.dim = prm->dim;
    a.tait = prm->tait;
    a.co = (float)prm->co; a.ro = (float)prm->ro; a.gamma = (float)prm->gamma;
    a.rho_out = rho; a.p_out = p; a.cs_out = cs;
    // the sorted state of the destination follows its own rho (and p, cs with
    // Tait); a density written to some other property leaves it untouched
    bool own = rho != nullptr && rho == D.view.rho &&
               (!prm->tait || (p == D.view.p && cs == D.view.cs));
    a.st_out = own ? D.st : nullptr;
    if (D.n == 0) return SPH_OK;
    int lpd = choose_lpd(ctx->grid);
    int blocks = blocks_for(D.n, lpd);
    int kx = ctx->grid.kx;
#define DISPATCH(KX_, L_) launch_density_t<KX_, L_>(a, blocks, ctx->stream)
    if (kx == 1) { if (lpd == 32) DISPATCH(1, 32); else if (lpd == 16) DISPATCH(1, 16); else DISPATCH(1, 8); }
    else if (kx == 2) { if (lpd == 32) DISPATCH(2, 32); else if (lpd == 16) DISPATCH(2, 16); else DISPATCH(2, 8); }
    else { if (lpd == 32) DISPATCH(3, 32); else if (lpd == 16) DISPATCH(3, 16); else DISPATCH(3, 8); }
#undef DISPATCH
    count_launch();
    SPH_LAUNCH_CHECK("k_density");
    return SPH_OK;
}

int launch_rates(sph_ctx *ctx, int dst, const sph_source_term *terms, int nterms,
                 const sph_rates_params *prm, double *const *acc, double *const *pos,
                 int accumulate) {
    if (!ctx->built) return set_error(SPH_ERR_STATE, "rates: no neighbour build");
    int na = (int)ctx->arrays.size();
    if (dst < 0 || dst >= na || nterms < 0 || nterms > SPH_MAX_SOURCES || !prm)
        return set_error(SPH_ERR_ARG, "rates: bad destination / sources");
    ArraySnap &D = ctx->arrays[dst];
    RatesArgs a{};
    a.g = ctx->grid;
    a.d = make_dest(D);
    a.nsrc = nterms;
    for (int i = 0; i < nterms; ++i) {
        int s = terms[i].src;
        if (s < 0 || s >= na) return set_error(SPH_ERR_ARG, "rates: bad source");
        if ((terms[i].flags & SPH_TERM_BFORCE) && !ctx->arrays[s].has_nrm)
            return set_error(SPH_ERR_ARG, "rates: boundary force source has no normals");
        a.s[i] = make_src(ctx->arrays[s]);
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
    if (D.n == 0) return SPH_OK;
    int lpd = choose_lpd(ctx->grid);
    int blocks = blocks_for(D.n, lpd);
    int kx = ctx->grid.kx;
#define DISPATCH(KX_, L_) launch_rates_t<KX_, L_>(a, blocks, ctx->stream)
    if (kx == 1) { if (lpd == 32) DISPATCH(1, 32); else if (lpd == 16) DISPATCH(1, 16); else DISPATCH(1, 8); }
    else if (kx == 2) { if (lpd == 32) DISPATCH(2, 32); else if (lpd == 16) DISPATCH(2, 16); else DISPATCH(2, 8); }
    else { if (lpd == 32) DISPATCH(3, 32); else if (lpd == 16) DISPATCH(3, 16); else DISPATCH(3, 8); }
#undef DISPATCH
    count_launch();
    SPH_LAUNCH_CHECK("k_rates");
    return SPH_OK;
}

}  // namespace sphgb
