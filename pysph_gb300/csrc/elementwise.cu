// Per-particle kernels (sm_103a): Tait equation of state, constant / velocity
// rates, the FP64 integrator update and FP64 invariant reductions.
#include <cuda_runtime.h>

#include <algorithm>

#include "sph_internal.cuh"

namespace sphgb {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ bool real_tag(const int64_t *tag, int64_t i) {
    return tag == nullptr || tag[i] == SPH_TAG_LOCAL_REAL;
}

// TaitEquation.eval_single (eos_funcs.pyx:105-116) in FP32 through
// log1p/expm1 of the density excess (relative accuracy kept as rho -> ro).
// gate: a launch inside a replayed step returns at once when a light
// refresh of that step found the neighbour lists stale (the host resumes the
// step after a full build)
__device__ __forceinline__ bool gated(const unsigned *gate) {
    return gate != nullptr && __ldg(gate) != 0u;
}

__global__ void k_tait(int64_t n, const double *rho, const int64_t *tag, float co, float ro,
                       float gamma, double *p, double *cs, const unsigned *gate) {
    if (gated(gate)) return;
    float B = co * co * ro / gamma;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (!real_tag(tag, i)) {
            p[i] = 0.0;
            cs[i] = 0.0;
            continue;
        }
        // the density excess in FP64: rho is within ~1e-3 of ro, where its
        // FP32 rounding would cost p about 1e-5 of its relative accuracy
        const float lr = log1pf((float)((rho[i] - (double)ro) / (double)ro));
        p[i] = (double)(B * expm1f(gamma * lr));
        cs[i] = (double)(co * expf(0.5f * (gamma - 1.f) * lr));
    }
}

struct ConstArgs {
    int kind, nout;
    double g[3];
    const double *vel[3];
    double *out[3];
};

// GravityForce (external_force.pyx:39-45) / PositionStepping (position_funcs.pyx:32-60)
__global__ void k_const(int64_t n, const int64_t *tag, ConstArgs a, const unsigned *gate) {
    if (gated(gate)) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        bool r = real_tag(tag, i);
        for (int c = 0; c < a.nout; ++c) {
            double v = a.kind == 0 ? a.g[c] : ld0(a.vel[c], i);
            a.out[c][i] = r ? v : 0.0;
        }
    }
}

struct AxpyArgs {
    sph_axpy_line l[SPH_MAX_AXPY_LINES];
    int nl;
};

// integrator.py:472-912: every line is rounded exactly like the NumPy
// expression it restates (left to right, no FMA contraction).
__global__ void k_axpy(int64_t n, const __grid_constant__ AxpyArgs a, const unsigned *gate) {
    if (gated(gate)) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        for (int k = 0; k < a.nl; ++k) {
            const sph_axpy_line &L = a.l[k];
            double b = L.base[i];
            double t;
            switch (L.mode) {
            case 0: {  // initial + 0.5*dt*(k1 + k2)
                double s = L.k2 ? __dadd_rn(L.k1[i], L.k2[i]) : L.k1[i];
                t = __dadd_rn(b, __dmul_rn(L.c1, s));
                break;
            }
            case 1:  // current + step*dt
                t = __dadd_rn(b, __dmul_rn(L.k1[i], L.c1));
                break;
            case 3:  // 2*current - initial
                t = __dsub_rn(__dmul_rn(2.0, b), L.k1[i]);
                break;
            case 4:  // current + 0.5*dt*(k2 - k1)
                t = __dadd_rn(b, __dmul_rn(L.c1, __dsub_rn(L.k2[i], L.k1[i])));
                break;
            case 5: {  // initial + dt/6*(k1 + 2*k2 + 2*k3 + k4)
                double s = __dadd_rn(L.k1[i], __dmul_rn(2.0, L.k2[i]));
                s = __dadd_rn(s, __dmul_rn(2.0, L.k3[i]));
                s = __dadd_rn(s, L.k4[i]);
                t = __dadd_rn(b, __dmul_rn(L.c1, s));
                break;
            }
            default:  // 2: copy
                t = b;
            }
            L.out[i] = t;
            if (L.save) L.save[i] = t;
        }
    }
}

constexpr int kRedBlocks = 2 * 152;

__global__ void k_invariants(sph_array_view a, double *part) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (!real_tag(a.tag, i)) continue;
        double m = a.m[i];
        double u = ld0(a.u, i), v = ld0(a.v, i), w = ld0(a.w, i);
        s[0] += m;
        s[1] += m * u;
        s[2] += m * v;
        s[3] += m * w;
        s[4] += 0.5 * m * (u * u + v * v + w * w);
        s[5] += 1.0;
    }
    __shared__ double sh[6][kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        double x = s[k];
        for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        if (lane == 0) sh[k][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double x = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x += sh[threadIdx.x][w];
        part[blockIdx.x * 6 + threadIdx.x] = x;
    }
}

__global__ void k_invariants_final(const double *part, int nb, double *out) {
    if (threadIdx.x < 6) {
        double x = 0;
        for (int b = 0; b < nb; ++b) x += part[b * 6 + threadIdx.x];
        out[threadIdx.x] = x;
    }
}

// ADKESmoothingUpdate.eval (adke_funcs.pyx:118-147), first pass: per-block
// FP64 sums of log(rhop) over LocalReal particles (fixed grid, fixed order).
__global__ void k_adke_logsum(int64_t n, const int64_t *tag, const double *rhop, double *part) {
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        if (real_tag(tag, i)) s = __dadd_rn(s, log(rhop[i]));
    __shared__ double sh[kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, off));
    if (lane == 0) sh[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x = __dadd_rn(x, sh[w]);
        part[blockIdx.x] = x;
    }
}

// second pass: every block sums the partials in the same order (the same g
// everywhere), then h = h0 k (g / rhop)^eps
__global__ void k_adke_h(int64_t n, const int64_t *tag, const double *rhop, const double *part,
                         int nb, double nreal, double h0k, double eps, double *h) {
    __shared__ double g_s;
    if (threadIdx.x == 0) {
        double x = 0.0;
        for (int b = 0; b < nb; ++b) x = __dadd_rn(x, part[b]);
        g_s = exp(__ddiv_rn(x, nreal));
    }
    __syncthreads();
    const double g = g_s;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        if (real_tag(tag, i)) h[i] = __dmul_rn(h0k, pow(__ddiv_rn(g, rhop[i]), eps));
}

// ADKEConductionCoeffUpdate.eval (adke_funcs.pyx:256-291)
__global__ void k_adke_q(int64_t nreal, const int64_t *tag, const double *cs, const double *h,
                         const double *div, double g1, double g2, double *q) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nreal;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (!real_tag(tag, i)) continue;
        const double ha = h[i], d = div[i];
        const double t = __dmul_rn(__dmul_rn(g2, ha), __dsub_rn(fabs(d), d));
        q[i] = __dmul_rn(__dadd_rn(__dmul_rn(g1, cs[i]), t), ha);
    }
}

}  // namespace

int launch_adke_smoothing(sph_ctx *ctx, int64_t n, int64_t nreal, const int64_t *tag,
                          const double *rhop, double h0, double k, double eps, double *h) {
    if (n < 0 || nreal < 0 || nreal > n || (n > 0 && (!rhop || !h)))
        return set_error(SPH_ERR_ARG, "adke_smoothing: bad arguments");
    if (n == 0) return SPH_OK;
    k_adke_logsum<<<kRedBlocks, kThreads, 0, ctx->stream>>>(n, tag, rhop, ctx->d_part);
    k_adke_h<<<grid_blocks(n, kThreads), kThreads, 0, ctx->stream>>>(
        n, tag, rhop, ctx->d_part, kRedBlocks, (double)nreal, h0 * k, eps, h);
    count_launch(2);
    SPH_LAUNCH_CHECK("k_adke_h");
    return SPH_OK;
}

int launch_adke_conduction(sph_ctx *ctx, int64_t nreal, const int64_t *tag, const double *cs,
                           const double *h, const double *div, double g1, double g2,
                           double *q) {
    if (nreal < 0 || (nreal > 0 && (!cs || !h || !div || !q)))
        return set_error(SPH_ERR_ARG, "adke_conduction: bad arguments");
    if (nreal == 0) return SPH_OK;
    k_adke_q<<<grid_blocks(nreal, kThreads), kThreads, 0, ctx->stream>>>(nreal, tag, cs, h, div,
                                                                       g1, g2, q);
    count_launch();
    SPH_LAUNCH_CHECK("k_adke_q");
    return SPH_OK;
}

int launch_tait(sph_ctx *ctx, int64_t n, const double *rho, const int64_t *tag, double co,
                double ro, double gamma, double *p, double *cs) {
    if (n < 0 || (n > 0 && (!rho || !p || !cs))) return set_error(SPH_ERR_ARG, "tait: bad arguments");
    if (n == 0) return SPH_OK;
    k_tait<<<grid_blocks(n, kThreads), kThreads, 0, ctx->stream>>>(n, rho, tag, (float)co, (float)ro,
                                                                  (float)gamma, p, cs, ctx->gate);
    count_launch();
    SPH_LAUNCH_CHECK("k_tait");
    return SPH_OK;
}

int launch_const_rates(sph_ctx *ctx, int kind, int64_t n, const int64_t *tag, const double *g3,
                       const double *u, const double *v, const double *w, int nout,
                       double *const *out) {
    if (n < 0 || nout < 1 || nout > 3 || (kind != 0 && kind != 1) || !out)
        return set_error(SPH_ERR_ARG, "const_rates: bad arguments");
    ConstArgs a{};
    a.kind = kind;
    a.nout = nout;
    for (int c = 0; c < 3; ++c) {
        a.g[c] = g3 ? g3[c] : 0.0;
        a.out[c] = c < nout ? out[c] : nullptr;
        if (c < nout && !a.out[c]) return set_error(SPH_ERR_ARG, "const_rates: null output");
    }
    a.vel[0] = u; a.vel[1] = v; a.vel[2] = w;
    if (n == 0) return SPH_OK;
    k_const<<<grid_blocks(n, kThreads), kThreads, 0, ctx->stream>>>(n, tag, a, ctx->gate);
    count_launch();
    SPH_LAUNCH_CHECK("k_const");
    return SPH_OK;
}

int launch_integrate(sph_ctx *ctx, int64_t n, const sph_axpy_line *lines, int nlines) {
    if (n < 0 || nlines < 0 || nlines > SPH_MAX_AXPY_LINES || (nlines > 0 && !lines))
        return set_error(SPH_ERR_ARG, "integrate: bad arguments");
    AxpyArgs a{};
    a.nl = nlines;
    for (int k = 0; k < nlines; ++k) {
        a.l[k] = lines[k];
        const sph_axpy_line &L = lines[k];
        if (L.mode < 0 || L.mode > 5) return set_error(SPH_ERR_ARG, "integrate: unknown line mode");
        if (!L.out || !L.base || (L.mode != 2 && !L.k1) || (L.mode == 4 && !L.k2) ||
            (L.mode == 5 && (!L.k2 || !L.k3 || !L.k4)))
            return set_error(SPH_ERR_ARG, "integrate: null array in a line");
    }
    if (n == 0 || nlines == 0) return SPH_OK;
    k_axpy<<<grid_blocks(n, kThreads), kThreads, 0, ctx->stream>>>(n, a, ctx->gate);
    count_launch();
    SPH_LAUNCH_CHECK("k_axpy");
    return SPH_OK;
}

int invariants(sph_ctx *ctx, const sph_array_view *a, double *out) {
    if (!a || !out) return set_error(SPH_ERR_ARG, "invariants: null argument");
    SPH_CUDA(cudaMemsetAsync(ctx->d_part, 0, sizeof(double) * (kRedBlocks * 6 + 8), ctx->stream));
    if (a->n > 0) {
        k_invariants<<<kRedBlocks, kThreads, 0, ctx->stream>>>(*a, ctx->d_part);
        count_launch();
    SPH_LAUNCH_CHECK("k_invariants");
    }
    k_invariants_final<<<1, 32, 0, ctx->stream>>>(ctx->d_part, kRedBlocks, ctx->d_part + kRedBlocks * 6);
    count_launch();
    SPH_LAUNCH_CHECK("k_invariants_final");
    SPH_CUDA(cudaMemcpyAsync(ctx->h_red, ctx->d_part + kRedBlocks * 6, 6 * sizeof(double),
                             cudaMemcpyDeviceToHost, ctx->stream));
    SPH_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < 6; ++k) out[k] = ctx->h_red[k];
    return SPH_OK;
}

int red_part_doubles() { return kRedBlocks * 6 + 8; }

}  // namespace sphgb
