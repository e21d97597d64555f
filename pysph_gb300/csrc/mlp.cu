// Learned momentum closure: the per-particle network 192 -> 128 -> 128 -> 2
// (GELU, tanh form) on the fifth-generation tensor cores.
//
// The reference has no learned part; the network stands in for the
// momentum pair loop (sph/funcs/pressure_funcs.pyx:40-91 and
// sph/funcs/viscosity_funcs.pyx:41-124) of a fluid array on itself.
//
// Operands: BF16 in shared memory, FP32 accumulation in tensor memory
// (tcgen05.mma kind::f16, M = 128 samples or hidden units, issued by one
// thread, completion through tcgen05.commit onto an mbarrier; the
// accumulator rows read back with tcgen05.ld by the warps that own their
// lane quarter).
//
//   k_mlp_fwd_tma  the forward, warp-specialised: TMA loads of X and the
//               weights into 128-byte-swizzled K-major atoms, one MMA warp,
//               16 epilogue warps (X W1^T -> +b1, GELU -> BF16 H1 in shared
//               memory -> H1 W2^T -> +b2, GELU -> h2 W3^T + b3 on the CUDA
//               cores, in packed FP32x2 arithmetic).  Training saves z1, z2
//               (FP32) and h1, h2 (BF16).
//   k_mlp_bwd_tma  the backward, warp-specialised: per tile z2 = h1 W2^T
//               + b2 recomputed, dz2 = (dy W3) * gelu'(z2), dh1 = dz2 W2,
//               dz1 = dh1 * gelu'(z1), and dW2 += dz2^T h1, dW1 += dz1^T x
//               accumulated in tensor memory over the CTA's tiles, the
//               sample-major tiles read as MN-major operands (no
//               transposes); a column of ones yields the bias gradients in
//               the same products.
//   k_mlp_fwd, k_mlp_bwd  the kernels these replace, kept to measure
//               against: plain staged loads in the canonical layout without
//               swizzle; operands transposed into 128-byte-swizzled staging
//               and the saved z2 read.
//   k_mlp_l3    third-layer gradients (FP32 CUDA cores).
//   k_mlp_reduce  fixed-order sum of the per-CTA partial gradients.
//   k_mlp_adam  Adam on the FP32 master parameters and the BF16 copies.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <mutex>

#include "sph_internal.cuh"

namespace sphgb {

namespace {

constexpr int NIN = SPH_MLP_NIN, NH = SPH_MLP_NH, NOUT = SPH_MLP_NOUT;
constexpr int OFF_W1 = SPH_MLP_OFF_W1, OFF_B1 = SPH_MLP_OFF_B1, OFF_W2 = SPH_MLP_OFF_W2,
              OFF_B2 = SPH_MLP_OFF_B2, OFF_W3 = SPH_MLP_OFF_W3, OFF_B3 = SPH_MLP_OFF_B3,
              NPARAM = SPH_MLP_NPARAM;
constexpr int TILE = 128;
constexpr int THREADS = 256;   // two warps per tensor-memory lane quarter
constexpr int L3_PART = NOUT * NH + NOUT;   // third-layer partial per block
constexpr int L3_ROWS = 1024;               // rows per third-layer block
constexpr int kMaxSpin = 1 << 22;           // bounded mbarrier wait
// per-CTA partial gradients of the backward: rows of PART_STRIDE floats
// (16-byte aligned)
constexpr int PART_STRIDE = (NPARAM + 3) & ~3;

// ---------------------------------------------------------------------------
// tcgen05 / mbarrier primitives (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading- and stride-
// dimension byte offsets (all >> 4), descriptor version 1 (bit 46), no
// swizzle (bits 61-63 = 0), base offset 0.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}
static_assert(idesc_bf16(128, 128) == 0x08200490u, "instruction descriptor layout");

__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Wait for phase `parity` of the barrier, at most kMaxSpin polls.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (int it = 0; it < kMaxSpin; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 16 consecutive FP32 accumulator columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// The same load without its wait: tmem_wait16 on the same registers before
// they are read (the registers are in-out operands of the wait, so nothing
// that reads them can be placed before it).
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait16(uint32_t (&r)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                   "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                   "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
}

// byte offset of element (r, k) of a K-major operand with kc = K/8 chunks per row
__device__ __forceinline__ uint32_t core_off(int r, int k, int kc) {
    return (uint32_t)(((((r >> 3) * kc) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// GELU in its tanh form (Hendrycks & Gimpel 2016):
//   gelu(z) = z/2 (1 + tanh(u)),  u = sqrt(2/pi) (z + 0.044715 z^3),
// with tanh(u) = 1 - 2 / (1 + e^(2u)) (saturates correctly for |u| large).
__device__ __forceinline__ float tanh_exp(float u) {
    return 1.f - __fdividef(2.f, 1.f + __expf(2.f * u));
}
__device__ __forceinline__ float gelu(float z) {
    const float u = 0.79788456080286536f * fmaf(0.044715f * z, z * z, z);
    return 0.5f * z * (1.f + tanh_exp(u));
}
// d gelu / dz = (1 + t)/2 + z/2 (1 - t^2) sqrt(2/pi) (1 + 3 * 0.044715 z^2)
__device__ __forceinline__ float dgelu(float z) {
    const float z2 = z * z;
    const float u = 0.79788456080286536f * fmaf(0.044715f * z, z2, z);
    const float t = tanh_exp(u);
    const float du = 0.79788456080286536f * fmaf(0.134145f, z2, 1.f);
    return fmaf(0.5f * z * (1.f - t * t), du, 0.5f * (1.f + t));
}

// The same derivative with s = 1 / (1 + e^(2u)) (so 1 + t = 2 (1 - s) and
// 1 - t^2 = 4 s (1 - s)):  d gelu / dz = (1 - s) (1 + 2 z s u'), the
// exponential and the reciprocal by the approximate special-function
// instructions (relative error near 2^-22; the backward's gradients are
// compared at 5e-3).
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float kGeluC = 0.79788456080286536f;             // sqrt(2/pi)
constexpr float kGeluE0 = 2.f * 1.4426950408889634f * kGeluC;   // 2u log2(e) = z (E0 + E1 z^2)
constexpr float kGeluE1 = kGeluE0 * 0.044715f;
constexpr float kGeluD0 = 2.f * kGeluC;                    // 2u' = D0 + D1 z^2
constexpr float kGeluD1 = kGeluD0 * 0.134145f;

// Pairs of FP32 values in one 64-bit register pair, for the packed FP32
// arithmetic of sm_100+ (add / sub / mul / fma .rn.f32x2: two lanes per
// instruction, each rounded like its scalar form).
__device__ __forceinline__ uint64_t f2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_split(uint64_t r, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// GELU of a pair, z/2 (1 + tanh(u)), with the special-function unit's
// tanh (tanh.approx.f32: one operation per value, against an exponential
// and a reciprocal, which made the special-function unit the forward
// epilogue's limiter).  Its error (about 2^-11 of |tanh u|) moves gelu by
// at most ~2.5e-4 |z|, below the BF16 rounding of the activations it
// feeds; tanh saturates to +-1, so both tails are exact in the limit.
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float kGeluU1 = kGeluC * 0.044715f;             // u = z (C + U1 z^2)
__device__ __forceinline__ uint64_t gelu2(uint64_t z) {
    const uint64_t u = mul2(z, fma2(mul2(z, z), f2(kGeluU1, kGeluU1), f2(kGeluC, kGeluC)));
    float u0, u1;
    f2_split(u, u0, u1);
    const uint64_t hz = mul2(z, f2(0.5f, 0.5f));
    return fma2(hz, f2(tanh_approx(u0), tanh_approx(u1)), hz);
}

// d gelu / dz of a pair in the sigmoid form: (1 - s) (1 + z (D0 + D1 z^2) s)
__device__ __forceinline__ uint64_t dgelu2(uint64_t z) {
    const uint64_t one = f2(1.f, 1.f);
    const uint64_t zz = mul2(z, z);
    const uint64_t ku = mul2(z, fma2(zz, f2(kGeluE1, kGeluE1), f2(kGeluE0, kGeluE0)));
    float k0, k1;
    f2_split(ku, k0, k1);
    const uint64_t d = add2(f2(ex2_approx(k0), ex2_approx(k1)), one);
    float d0, d1;
    f2_split(d, d0, d1);
    const uint64_t sg = f2(rcp_approx(d0), rcp_approx(d1));
    const uint64_t zq = mul2(z, fma2(zz, f2(kGeluD1, kGeluD1), f2(kGeluD0, kGeluD0)));
    return mul2(sub2(one, sg), fma2(zq, sg, one));
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// Copy a row-major [rows][K] BF16 matrix into the K-major core layout.
// Eight consecutive threads take the eight rows of one core matrix (one
// 16-byte chunk each) so their shared stores hit distinct banks.
__device__ __forceinline__ void load_operand(uint8_t *dst, const uint16_t *src, int rows, int K) {
    const int kc = K / 8;
    for (int c = threadIdx.x; c < rows * kc; c += blockDim.x) {
        const int r8 = c & 7, rest = c >> 3;
        const int k8 = rest % kc, rg = rest / kc;
        const int r = rg * 8 + r8;
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(src + (int64_t)r * K + k8 * 8));
        *reinterpret_cast<uint4 *>(dst + core_off(r, k8 * 8, kc)) = v;
    }
}

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
constexpr uint32_t F_W1 = 0;
constexpr uint32_t F_W2 = F_W1 + NH * NIN * 2;      // 49152
constexpr uint32_t F_X = F_W2 + NH * NH * 2;        // 81920
constexpr uint32_t F_H1 = F_X + TILE * NIN * 2;     // 131072
constexpr uint32_t F_W3 = F_H1 + TILE * NH * 2;     // 163840: float [2][128]
constexpr uint32_t F_B1 = F_W3 + NOUT * NH * 4;     // float [128]
constexpr uint32_t F_B2 = F_B1 + NH * 4;            // float [128]
constexpr uint32_t F_B3 = F_B2 + NH * 4;            // float [2] (+pad)
constexpr uint32_t F_YP = F_B3 + 16;                // float2 [128]: upper-half outputs
constexpr uint32_t F_BAR = F_YP + TILE * 8;         // mbarrier (8 B)
constexpr uint32_t F_SLOT = F_BAR + 8;              // tensor-memory address
constexpr uint32_t F_BYTES = F_SLOT + 8;
constexpr uint32_t F_TMEM_COLS = 256;               // z1 at 0, z2 at 128

struct MlpDev {
    const float *params;
    const uint16_t *w1, *w2, *w2t, *w3;
};

__global__ void __launch_bounds__(THREADS, 1)
    k_mlp_fwd(const MlpDev W, const uint16_t *__restrict__ x, int64_t n, float *__restrict__ y,
              float *__restrict__ z1s, float *__restrict__ z2s, uint16_t *__restrict__ h1s,
              uint16_t *__restrict__ h2s, unsigned *err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    // warps w and w + 4 read the same 32 tensor-memory lanes (tile rows),
    // each one half of the accumulator columns
    const int q = warp & 3, ch = warp >> 2;
    const int row = q * 32 + lane;
    const int cbeg = ch * (NH / 2), cend = cbeg + NH / 2;
    float *w3f = reinterpret_cast<float *>(sm + F_W3);
    float2 *yp = reinterpret_cast<float2 *>(sm + F_YP);
    float *b1f = reinterpret_cast<float *>(sm + F_B1);
    float *b2f = reinterpret_cast<float *>(sm + F_B2);
    float *b3f = reinterpret_cast<float *>(sm + F_B3);
    const uint32_t bar = smem_u32(sm + F_BAR);
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + F_SLOT);

    load_operand(sm + F_W1, W.w1, NH, NIN);
    load_operand(sm + F_W2, W.w2, NH, NH);
    for (int i = t; i < NOUT * NH; i += THREADS) w3f[i] = __uint_as_float((uint32_t)W.w3[i] << 16);
    for (int i = t; i < NH; i += THREADS) {
        b1f[i] = W.params[OFF_B1 + i];
        b2f[i] = W.params[OFF_B2 + i];
    }
    if (t < NOUT) b3f[t] = W.params[OFF_B3 + t];
    if (warp == 0) tmem_alloc(smem_u32(slot), F_TMEM_COLS);
    if (t == 0) mbar_init(bar, 1);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *slot;
    const uint32_t lane_base = (uint32_t)(q * 32) << 16;
    const uint32_t sX = smem_u32(sm + F_X), sW1 = smem_u32(sm + F_W1);
    const uint32_t sH1 = smem_u32(sm + F_H1), sW2 = smem_u32(sm + F_W2);
    uint32_t phase = 0;
    bool ok = true;

    const int64_t ntiles = (n + TILE - 1) / TILE;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t row0 = tile * TILE;
        // X tile (rows beyond n are zeros)
        for (int c = t; c < TILE * (NIN / 8); c += THREADS) {
            const int r8 = c & 7, rest = c >> 3;
            const int k8 = rest % (NIN / 8), rg = rest / (NIN / 8);
            const int r = rg * 8 + r8;
            const int64_t gr = row0 + r;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (gr < n) v = __ldg(reinterpret_cast<const uint4 *>(x + gr * NIN + k8 * 8));
            *reinterpret_cast<uint4 *>(sm + F_X + core_off(r, k8 * 8, NIN / 8)) = v;
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
#pragma unroll
            for (int s = 0; s < NIN / 16; ++s)
                mma_bf16(tbase, sdesc(sX + s * 256, 128, (NIN / 8) * 128),
                         sdesc(sW1 + s * 256, 128, (NIN / 8) * 128), idesc_bf16(128, NH), s > 0);
            mma_commit(bar);
        }
        ok = mbar_wait(bar, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) break;
        tc_fence_after();

        const int64_t grow = row0 + row;
        const bool valid = grow < n;
#pragma unroll 1
        for (int c0 = cbeg; c0 < cend; c0 += 16) {
            float v[16];
            tmem_ld16(tbase + lane_base + c0, v);
            uint32_t hw[8];
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] += b1f[c0 + i];
#pragma unroll
            for (int i = 0; i < 8; ++i) hw[i] = pack2(gelu(v[2 * i]), gelu(v[2 * i + 1]));
            *reinterpret_cast<uint4 *>(sm + F_H1 + core_off(row, c0, NH / 8)) =
                make_uint4(hw[0], hw[1], hw[2], hw[3]);
            *reinterpret_cast<uint4 *>(sm + F_H1 + core_off(row, c0 + 8, NH / 8)) =
                make_uint4(hw[4], hw[5], hw[6], hw[7]);
            if (valid && z1s) {
                float4 *zp = reinterpret_cast<float4 *>(z1s + grow * NH + c0);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    zp[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
            if (valid && h1s) {
                uint4 *hp = reinterpret_cast<uint4 *>(h1s + grow * NH + c0);
                hp[0] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                hp[1] = make_uint4(hw[4], hw[5], hw[6], hw[7]);
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
#pragma unroll
            for (int s = 0; s < NH / 16; ++s)
                mma_bf16(tbase + 128, sdesc(sH1 + s * 256, 128, (NH / 8) * 128),
                         sdesc(sW2 + s * 256, 128, (NH / 8) * 128), idesc_bf16(128, NH), s > 0);
            mma_commit(bar);
        }
        ok = mbar_wait(bar, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) break;
        tc_fence_after();

        float y0 = 0.f, y1 = 0.f;
#pragma unroll 1
        for (int c0 = cbeg; c0 < cend; c0 += 16) {
            float v[16];
            tmem_ld16(tbase + 128 + lane_base + c0, v);
            uint32_t hw[8];
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] += b2f[c0 + i];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                hw[i] = pack2(gelu(v[2 * i]), gelu(v[2 * i + 1]));
                const float ha = bf_lo(hw[i]), hb = bf_hi(hw[i]);
                const int c = c0 + 2 * i;
                y0 = fmaf(ha, w3f[c], y0);
                y0 = fmaf(hb, w3f[c + 1], y0);
                y1 = fmaf(ha, w3f[NH + c], y1);
                y1 = fmaf(hb, w3f[NH + c + 1], y1);
            }
            if (valid && z2s) {
                float4 *zp = reinterpret_cast<float4 *>(z2s + grow * NH + c0);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    zp[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
            if (valid && h2s) {
                uint4 *hp = reinterpret_cast<uint4 *>(h2s + grow * NH + c0);
                hp[0] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                hp[1] = make_uint4(hw[4], hw[5], hw[6], hw[7]);
            }
        }
        if (ch == 1) yp[row] = make_float2(y0, y1);
        __syncthreads();
        if (ch == 0 && valid) {
            const float2 o = yp[row];
            y[grow * 2] = b3f[0] + (y0 + o.x);
            y[grow * 2 + 1] = b3f[1] + (y1 + o.y);
        }
        tc_fence_before();
        __syncthreads();
    }
    if (!ok && t == 0) atomicOr(err, SPH_EFLAG_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tbase, F_TMEM_COLS);
    }
}

// ---------------------------------------------------------------------------
// forward, warp-specialised: tiles and weights brought in by the tensor
// memory access unit (TMA) into 128-byte-swizzled shared memory, two sample
// tiles in flight, the first layer's accumulator double-buffered in tensor
// memory so that a tile's first product runs while the previous tile's
// epilogues do
// ---------------------------------------------------------------------------
// Shared memory, from a 1024-byte aligned base: operands in the canonical
// K-major layout with 128-byte swizzling, in atoms of 128 rows x 64 BF16
// (16 KB; the box one TMA load writes): W1 3 atoms (K = 192), W2 2, X two
// stages of 3, H1 2 (written by the epilogue in the same layout).
constexpr uint32_t ATOM = 128 * 128;
constexpr uint32_t G_W1 = 0;
constexpr uint32_t G_W2 = G_W1 + 3 * ATOM;
constexpr uint32_t G_X = G_W2 + 2 * ATOM;
constexpr uint32_t G_H1 = G_X + 2 * 3 * ATOM;
constexpr uint32_t G_B1 = G_H1 + 2 * ATOM;          // float [128]
constexpr uint32_t G_B2 = G_B1 + NH * 4;            // float [128]
constexpr uint32_t G_W3 = G_B2 + NH * 4;            // float [2][128]
constexpr uint32_t G_B3 = G_W3 + NOUT * NH * 4;     // float [2] (+pad)
// epilogue warps: four per lane quarter of the accumulators, each a quarter
// of the columns (four warps per scheduler to hide the epilogue's latency)
constexpr int G_EPI = 16;
constexpr int G_COLS = NH / (G_EPI / 4);            // 32 columns per epilogue warp
constexpr uint32_t G_YP = G_B3 + 16;                // float2 [2 tile parities][4 parts][128]
constexpr uint32_t G_BAR = G_YP + 2 * (G_EPI / 4) * TILE * 8;
// mbarriers: weights; X stage full / empty; first accumulator full / empty
// (two each); H1 full / empty; second accumulator full / empty (two each);
// output partials of the column parts written (two, by tile parity)
enum GBar { GB_W = 0, GB_XF0, GB_XF1, GB_XE0, GB_XE1, GB_A1F0, GB_A1F1, GB_A1E0, GB_A1E1,
            GB_HF, GB_HE, GB_A2F0, GB_A2F1, GB_A2E0, GB_A2E1, GB_Y0, GB_Y1, GB_N };
constexpr uint32_t G_SLOT = G_BAR + GB_N * 8;        // tensor-memory address
constexpr uint32_t G_ABORT = G_SLOT + 4;            // a bounded wait gave up
constexpr uint32_t G_END = G_ABORT + 4;
constexpr uint32_t G_BYTES = G_END + 1024;          // + alignment of the base
constexpr int G_THREADS = 32 * (2 + G_EPI);        // producer, MMA, 16 epilogue warps
constexpr uint32_t G_TMEM_COLS = 512;               // acc1 at 0 and 128, acc2 at 256 and 384
constexpr uint32_t G_XBYTES = 3 * ATOM;

// Shared-memory matrix descriptor, K-major with 128-byte swizzling: start
// address >> 4, leading offset 16 B (unused for swizzled K-major), stride
// offset 1024 B (eight 128-byte rows), version 1 (bit 46), swizzle mode 2
// (bits 61-63).  A K step of 16 BF16 advances the start by 32 B within an
// atom.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// 2D tile load (x = column in elements, a multiple of 64, y = row) into
// shared memory, completing on the mbarrier's transaction count.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, uint32_t mbar,
                                            int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(mbar), "r"(x), "r"(y)
        : "memory");
}

// Bounded wait that also gives up when another role has (the abort word).
__device__ __forceinline__ bool gwait(uint32_t mbar, uint32_t parity, volatile int *abort) {
    for (int it = 0; it < kMaxSpin; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255) == 255 && *abort) return false;
    }
    *abort = 1;
    return false;
}

// Byte offset of the 16-byte chunk (row r, columns 8c .. 8c + 7) of a
// 128-byte-swizzled atom.
__device__ __forceinline__ uint32_t sw128_off(int r, int c) {
    return (uint32_t)(r * 128 + ((c ^ (r & 7)) << 4));
}

struct MlpMaps {
    CUtensorMap x, w1, w2;
};

__global__ void __launch_bounds__(G_THREADS, 1)
    k_mlp_fwd_tma(const __grid_constant__ MlpMaps maps, const float *__restrict__ params,
                  const uint16_t *__restrict__ w3b, int64_t n, float *__restrict__ y,
                  float *__restrict__ z1s, float *__restrict__ z2s, uint16_t *__restrict__ h1s,
                  uint16_t *__restrict__ h2s, unsigned *err) {
    extern __shared__ __align__(1024) uint8_t gsm_raw[];
    const uint32_t raw = smem_u32(gsm_raw);
    uint8_t *sm = gsm_raw + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t sbase = smem_u32(sm);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    float *b1f = reinterpret_cast<float *>(sm + G_B1);
    float *b2f = reinterpret_cast<float *>(sm + G_B2);
    float *w3f = reinterpret_cast<float *>(sm + G_W3);
    float *b3f = reinterpret_cast<float *>(sm + G_B3);
    float2 *yp = reinterpret_cast<float2 *>(sm + G_YP);
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + G_SLOT);
    volatile int *abort = reinterpret_cast<volatile int *>(sm + G_ABORT);
    auto bar = [&](int i) { return sbase + G_BAR + 8u * (uint32_t)i; };

    for (int i = t; i < NH; i += G_THREADS) {
        b1f[i] = params[OFF_B1 + i];
        b2f[i] = params[OFF_B2 + i];
    }
    for (int i = t; i < NOUT * NH; i += G_THREADS) w3f[i] = __uint_as_float((uint32_t)w3b[i] << 16);
    if (t < NOUT) b3f[t] = params[OFF_B3 + t];
    if (t == 0) {
        *abort = 0;
        mbar_init(bar(GB_W), 1);
        mbar_init(bar(GB_XF0), 1);
        mbar_init(bar(GB_XF1), 1);
        mbar_init(bar(GB_XE0), 1);
        mbar_init(bar(GB_XE1), 1);
        mbar_init(bar(GB_A1F0), 1);
        mbar_init(bar(GB_A1F1), 1);
        mbar_init(bar(GB_A1E0), G_EPI);
        mbar_init(bar(GB_A1E1), G_EPI);
        mbar_init(bar(GB_HF), G_EPI);
        mbar_init(bar(GB_HE), 1);
        mbar_init(bar(GB_A2F0), 1);
        mbar_init(bar(GB_A2F1), 1);
        mbar_init(bar(GB_A2E0), G_EPI);
        mbar_init(bar(GB_A2E1), G_EPI);
        mbar_init(bar(GB_Y0), G_EPI);
        mbar_init(bar(GB_Y1), G_EPI);
    }
    if (warp == 0) tmem_alloc(smem_u32(slot), G_TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *slot;
    const int64_t ntiles = (n + TILE - 1) / TILE;
    // this CTA's tiles: blockIdx.x, + gridDim.x, ...
    const int mine = ntiles > blockIdx.x ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;

    if (warp == 0) {
        // producer: weights once, then the sample tiles through two stages
        if (lane == 0) {
            mbar_expect_tx(bar(GB_W), 5 * ATOM);
            for (int a = 0; a < 3; ++a) tma_load_2d(sbase + G_W1 + a * ATOM, &maps.w1, bar(GB_W), 64 * a, 0);
            for (int a = 0; a < 2; ++a) tma_load_2d(sbase + G_W2 + a * ATOM, &maps.w2, bar(GB_W), 64 * a, 0);
            for (int i = 0; i < mine; ++i) {
                const int s = i & 1;
                if (!gwait(bar(GB_XE0 + s), ((i >> 1) + 1) & 1, abort)) break;
                const int row0 = (int)((blockIdx.x + (int64_t)i * gridDim.x) * TILE);
                mbar_expect_tx(bar(GB_XF0 + s), G_XBYTES);
                for (int a = 0; a < 3; ++a)
                    tma_load_2d(sbase + G_X + (s * 3 + a) * ATOM, &maps.x, bar(GB_XF0 + s), 64 * a, row0);
            }
            // every load issued has landed before the CTA may exit
            for (int i = (mine > 2 ? mine - 2 : 0); i < mine; ++i)
                gwait(bar(GB_XF0 + (i & 1)), (i >> 1) & 1, abort);
            gwait(bar(GB_W), 0, abort);
        }
    } else if (warp == 1) {
        // MMA issue: the first layer of tile i + 1 before the second of tile i
        if (lane == 0) {
            constexpr uint32_t ID = idesc_bf16(128, NH);
            bool ok = gwait(bar(GB_W), 0, abort);
            auto first_layer = [&](int i) -> bool {
                const int s = i & 1;
                if (!gwait(bar(GB_XF0 + s), (i >> 1) & 1, abort)) return false;
                if (!gwait(bar(GB_A1E0 + s), ((i >> 1) + 1) & 1, abort)) return false;
                tc_fence_after();
#pragma unroll
                for (int k = 0; k < NIN / 16; ++k) {
                    const uint32_t a = sbase + G_X + (s * 3 + (k >> 2)) * ATOM + (k & 3) * 32;
                    const uint32_t b = sbase + G_W1 + (k >> 2) * ATOM + (k & 3) * 32;
                    mma_bf16(tbase + s * 128, sdesc_sw128(a), sdesc_sw128(b), ID, k > 0);
                }
                mma_commit(bar(GB_XE0 + s));
                mma_commit(bar(GB_A1F0 + s));
                return true;
            };
            if (ok && mine > 0) ok = first_layer(0);
            for (int i = 0; ok && i < mine; ++i) {
                if (i + 1 < mine && !first_layer(i + 1)) break;
                const int s2 = i & 1;
                if (!gwait(bar(GB_HF), i & 1, abort)) break;
                if (!gwait(bar(GB_A2E0 + s2), ((i >> 1) + 1) & 1, abort)) break;
                tc_fence_after();
#pragma unroll
                for (int k = 0; k < NH / 16; ++k) {
                    const uint32_t a = sbase + G_H1 + (k >> 2) * ATOM + (k & 3) * 32;
                    const uint32_t b = sbase + G_W2 + (k >> 2) * ATOM + (k & 3) * 32;
                    mma_bf16(tbase + 256 + 128 * s2, sdesc_sw128(a), sdesc_sw128(b), ID, k > 0);
                }
                mma_commit(bar(GB_HE));
                mma_commit(bar(GB_A2F0 + s2));
            }
        }
    } else {
        // epilogues: lane quarter q of the accumulators, column part hf
        const int q = warp & 3, hf = (warp - 2) >> 2;
        const int row = q * 32 + lane;
        const uint32_t lane_base = (uint32_t)(q * 32) << 16;
        const int cb = hf * G_COLS;
        // a wait every lane of the warp agrees on (the tensor-memory loads
        // after it are warp-wide)
        auto wwait = [&](int k, int parity) {
            return __all_sync(0xffffffffu, gwait(bar(k), (uint32_t)parity & 1u, abort)) != 0;
        };
        // layer 1 of tile i: acc1[i % 2] + b1, GELU -> H1 (and the saved values)
        auto layer1 = [&](int i) -> bool {
            const int s = i & 1;
            const int64_t grow = (blockIdx.x + (int64_t)i * gridDim.x) * TILE + row;
            const bool valid = grow < n;
            // layer 1: acc1[s] + b1, GELU -> H1 (and the saved values)
            if (!wwait(GB_A1F0 + s, (i >> 1) & 1)) return false;
            tc_fence_after();
            uint32_t hw[G_COLS / 2];
            // the second chunk's load in flight while the first is computed
            uint32_t rr[2][16];
            tmem_ld16_async(tbase + s * 128 + lane_base + cb, rr[0]);
            tmem_wait16(rr[0]);
            tmem_ld16_async(tbase + s * 128 + lane_base + cb + 16, rr[1]);
#pragma unroll
            for (int c = 0; c < G_COLS / 16; ++c) {
                if (c == 1) tmem_wait16(rr[1]);
                float v[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) v[e] = __uint_as_float(rr[c][e]);
                // + b1 and GELU, two columns per packed instruction
                uint64_t z[8];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float4 bb = *reinterpret_cast<const float4 *>(b1f + cb + 16 * c + 4 * e);
                    z[2 * e] = add2(f2(v[4 * e], v[4 * e + 1]), f2(bb.x, bb.y));
                    z[2 * e + 1] = add2(f2(v[4 * e + 2], v[4 * e + 3]), f2(bb.z, bb.w));
                }
                if (valid && z1s) {
                    float4 *zp = reinterpret_cast<float4 *>(z1s + grow * NH + cb + 16 * c);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        float a0, a1, a2, a3;
                        f2_split(z[2 * e], a0, a1);
                        f2_split(z[2 * e + 1], a2, a3);
                        zp[e] = make_float4(a0, a1, a2, a3);
                    }
                }
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    float g0, g1;
                    f2_split(gelu2(z[e]), g0, g1);
                    hw[8 * c + e] = pack2(g0, g1);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(GB_A1E0 + s));
            // H1 is free once the second layer of the previous tile has read it
            if (!wwait(GB_HE, (i + 1) & 1)) return false;
            // columns cb .. cb + 31: atom cb / 64, chunks (cb % 64) / 8 + c
#pragma unroll
            for (int c = 0; c < G_COLS / 8; ++c)
                *reinterpret_cast<uint4 *>(sm + G_H1 + (cb >> 6) * ATOM +
                                           sw128_off(row, ((cb & 63) >> 3) + c)) =
                    make_uint4(hw[4 * c], hw[4 * c + 1], hw[4 * c + 2], hw[4 * c + 3]);
            if (valid && h1s) {
                uint4 *hp = reinterpret_cast<uint4 *>(h1s + grow * NH + cb);
#pragma unroll
                for (int c = 0; c < G_COLS / 8; ++c)
                    hp[c] = make_uint4(hw[4 * c], hw[4 * c + 1], hw[4 * c + 2], hw[4 * c + 3]);
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(GB_HF));
            return true;
        };
        // layer 2 of tile i: acc2[i % 2] + b2, GELU, the output layer
        auto layer2 = [&](int i) -> bool {
            const int s = i & 1;
            const int64_t grow = (blockIdx.x + (int64_t)i * gridDim.x) * TILE + row;
            const bool valid = grow < n;
            // layer 2: acc2 + b2, GELU, then the output layer on the CUDA cores
            const int s2 = i & 1;
            if (!wwait(GB_A2F0 + s2, (i >> 1) & 1)) return false;
            tc_fence_after();
            // the output layer in packed pairs: (y0 over even, odd columns), (y1 ...)
            uint64_t ya = f2(0.f, 0.f), yb = f2(0.f, 0.f);
            uint32_t rr2[2][16];
            tmem_ld16_async(tbase + 256 + 128 * s2 + lane_base + cb, rr2[0]);
            tmem_wait16(rr2[0]);
            tmem_ld16_async(tbase + 256 + 128 * s2 + lane_base + cb + 16, rr2[1]);
#pragma unroll
            for (int c = 0; c < G_COLS / 16; ++c) {
                if (c == 1) tmem_wait16(rr2[1]);
                float v[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) v[e] = __uint_as_float(rr2[c][e]);
                uint32_t w2w[8];
                uint64_t z[8];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float4 bb = *reinterpret_cast<const float4 *>(b2f + cb + 16 * c + 4 * e);
                    z[2 * e] = add2(f2(v[4 * e], v[4 * e + 1]), f2(bb.x, bb.y));
                    z[2 * e + 1] = add2(f2(v[4 * e + 2], v[4 * e + 3]), f2(bb.z, bb.w));
                }
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    float g0, g1;
                    f2_split(gelu2(z[e]), g0, g1);
                    w2w[e] = pack2(g0, g1);
                    const int j = cb + 16 * c + 2 * e;
                    const uint64_t h = f2(bf_lo(w2w[e]), bf_hi(w2w[e]));
                    ya = fma2(h, *reinterpret_cast<const uint64_t *>(w3f + j), ya);
                    yb = fma2(h, *reinterpret_cast<const uint64_t *>(w3f + NH + j), yb);
                }
                if (valid && z2s) {
                    float4 *zp = reinterpret_cast<float4 *>(z2s + grow * NH + cb + 16 * c);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        float a0, a1, a2, a3;
                        f2_split(z[2 * e], a0, a1);
                        f2_split(z[2 * e + 1], a2, a3);
                        zp[e] = make_float4(a0, a1, a2, a3);
                    }
                }
                if (valid && h2s) {
                    uint4 *hp = reinterpret_cast<uint4 *>(h2s + grow * NH + cb + 16 * c);
                    hp[0] = make_uint4(w2w[0], w2w[1], w2w[2], w2w[3]);
                    hp[1] = make_uint4(w2w[4], w2w[5], w2w[6], w2w[7]);
                }
            }
            float y0, y1;
            {
                float a0, a1, b0, b1;
                f2_split(ya, a0, a1);
                f2_split(yb, b0, b1);
                y0 = a0 + a1;
                y1 = b0 + b1;
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(GB_A2E0 + s2));
            // the column parts of a row meet: all write their partial, the
            // first part adds them in a fixed order (the partials alternate
            // by tile parity; a tile's H1 barrier orders the reuse)
            constexpr int NP = G_EPI / 4;
            yp[(s * NP + hf) * TILE + row] = make_float2(y0, y1);
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(GB_Y0 + s));
            if (hf == 0) {
                if (!wwait(GB_Y0 + s, (i >> 1) & 1)) return false;
                if (valid) {
#pragma unroll
                    for (int pp = 1; pp < NP; ++pp) {
                        const float2 o = yp[(s * NP + pp) * TILE + row];
                        y0 += o.x;
                        y1 += o.y;
                    }
                    y[grow * 2] = b3f[0] + y0;
                    y[grow * 2 + 1] = b3f[1] + y1;
                }
            }
            return true;
        };
        // the first layer of tile i + 1 before the second of tile i: its math
        // runs while the tensor cores compute the second product of tile i
        if (mine > 0 && layer1(0)) {
            for (int i = 0; i < mine; ++i) {
                if (i + 1 < mine && !layer1(i + 1)) break;
                if (!layer2(i)) break;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (*abort && t == 0) atomicOr(err, SPH_EFLAG_TIMEOUT);
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tbase, G_TMEM_COLS);
    }
}

// ---------------------------------------------------------------------------
// backward
// ---------------------------------------------------------------------------
// Operands in the K-major layout with 128-byte swizzling (as the TMA forward
// kernel's): an operand of R rows keeps K in atom columns of 64 BF16, each
// R x 128 B; within one, row r's 16-byte chunk c sits at chunk c ^ (r % 8).
// The transposed operands are written one 2-byte element per thread (the
// thread's sample is the K index): the swizzle spreads a warp's 32 samples
// over four chunks of the row, so a store takes one wavefront.
__device__ __forceinline__ uint32_t sw_off(int r, int k, int rows) {
    return (uint32_t)((k >> 6) * rows * 128 + r * 128 + ((((k & 63) >> 3) ^ (r & 7)) << 4) +
                      ((k & 7) << 1));
}

// Start address of K step s (16 BF16) of an operand of R rows.
__device__ __forceinline__ uint32_t sw_kstep(uint32_t base, int s, int rows) {
    return base + (uint32_t)((s >> 2) * rows * 128 + (s & 3) * 32);
}

// Copy a row-major [rows][K] BF16 matrix into the swizzled layout.
__device__ __forceinline__ void load_operand_sw(uint8_t *dst, const uint16_t *src, int rows, int K) {
    const int kc = K / 8;
    for (int c = threadIdx.x; c < rows * kc; c += blockDim.x) {
        const int r = c / kc, k8 = c % kc;
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(src + (int64_t)r * K + k8 * 8));
        *reinterpret_cast<uint4 *>(dst + sw_off(r, k8 * 8, rows)) = v;
    }
}

constexpr int H1T_ROWS = NH + 16;    // h1^T plus a row of ones (bias) and zero rows
constexpr int XT_ROWS = NIN + 16;    // x^T plus a row of ones and zero rows
constexpr uint32_t B_A1 = 0;                              // dz2 [b][j]
constexpr uint32_t B_A2 = B_A1 + TILE * NH * 2;           // dz2^T, then dz1^T [j][b]
constexpr uint32_t B_H1T = B_A2 + NH * TILE * 2;          // [i][b], 144 rows
constexpr uint32_t B_XT = B_H1T + H1T_ROWS * TILE * 2;    // [m][b], 208 rows
constexpr uint32_t B_W2T = B_XT + XT_ROWS * TILE * 2;     // W2^T [i][j]
constexpr uint32_t B_W3 = B_W2T + NH * NH * 2;            // float [2][128]
constexpr uint32_t B_RED = B_W3 + NOUT * NH * 4;          // float [8] loss per warp
constexpr uint32_t B_BAR = B_RED + 32;
constexpr uint32_t B_SLOT = B_BAR + 8;
constexpr uint32_t B_BYTES = B_SLOT + 8 + 1024;           // + alignment of the base
constexpr uint32_t T_DH1 = 0, T_DW2 = 128, T_DW1 = 288;    // tensor-memory columns
constexpr uint32_t B_TMEM_COLS = 512;
static_assert(T_DW2 + H1T_ROWS <= T_DW1 && T_DW1 + XT_ROWS <= B_TMEM_COLS, "tensor memory plan");

__global__ void __launch_bounds__(THREADS, 1)
    k_mlp_bwd(const MlpDev W, const uint16_t *__restrict__ x, const uint16_t *__restrict__ h1s,
              const float *__restrict__ z1s, const float *__restrict__ z2s,
              const float *__restrict__ y, const float *__restrict__ target, int64_t n,
              float inv_count, float *__restrict__ dy_out, float *__restrict__ part,
              float *__restrict__ part_loss, unsigned *err) {
    extern __shared__ __align__(1024) uint8_t bsm_raw[];
    const uint32_t raw = smem_u32(bsm_raw);
    uint8_t *sm = bsm_raw + (((raw + 1023u) & ~1023u) - raw);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    // row = sample (and tensor-memory lane); the two warps of a lane quarter
    // split the columns
    const int q = warp & 3, ch = warp >> 2;
    const int row = q * 32 + lane;
    float *w3f = reinterpret_cast<float *>(sm + B_W3);
    float *red = reinterpret_cast<float *>(sm + B_RED);
    const uint32_t bar = smem_u32(sm + B_BAR);
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + B_SLOT);

    load_operand_sw(sm + B_W2T, W.w2t, NH, NH);
    for (int i = t; i < NOUT * NH; i += THREADS) w3f[i] = __uint_as_float((uint32_t)W.w3[i] << 16);
    // the constant rows: ones at h1^T row 128 and x^T row 192, zeros below
    for (int i = t; i < 16 * TILE; i += THREADS) {
        const int r = i / TILE, b = i % TILE;
        const __nv_bfloat16 one = __float2bfloat16_rn(r == 0 ? 1.f : 0.f);
        *reinterpret_cast<__nv_bfloat16 *>(sm + B_H1T + sw_off(NH + r, b, H1T_ROWS)) = one;
        *reinterpret_cast<__nv_bfloat16 *>(sm + B_XT + sw_off(NIN + r, b, XT_ROWS)) = one;
    }
    if (warp == 0) tmem_alloc(smem_u32(slot), B_TMEM_COLS);
    if (t == 0) mbar_init(bar, 1);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *slot;
    const uint32_t lane_base = (uint32_t)(q * 32) << 16;
    const uint32_t sA1 = smem_u32(sm + B_A1), sA2 = smem_u32(sm + B_A2);
    const uint32_t sH1T = smem_u32(sm + B_H1T), sXT = smem_u32(sm + B_XT);
    const uint32_t sW2T = smem_u32(sm + B_W2T);
    uint32_t phase = 0;
    bool ok = true, first = true;
    float loss = 0.f;

    const int64_t ntiles = (n + TILE - 1) / TILE;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t b = tile * TILE + row;
        const bool valid = b < n;
        float d0 = 0.f, d1 = 0.f;
        if (valid) {
            const float e0 = y[b * 2] - target[b * 2], e1 = y[b * 2 + 1] - target[b * 2 + 1];
            d0 = e0 * inv_count;
            d1 = e1 * inv_count;
            if (ch == 0) {
                loss += e0 * e0 + e1 * e1;
                dy_out[b * 2] = d0;
                dy_out[b * 2 + 1] = d1;
            }
        }
        // dz2 = (dy W3) * gelu'(z2): row `row` of A1, column `row` of A2
        // (loops unrolled by four so that four rows' loads are in flight)
#pragma unroll 4
        for (int j0 = ch * (NH / 2); j0 < (ch + 1) * (NH / 2); j0 += 8) {
            float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (valid) {
                const float4 a = *reinterpret_cast<const float4 *>(z2s + b * NH + j0);
                const float4 c = *reinterpret_cast<const float4 *>(z2s + b * NH + j0 + 4);
                z[0] = a.x; z[1] = a.y; z[2] = a.z; z[3] = a.w;
                z[4] = c.x; z[5] = c.y; z[6] = c.z; z[7] = c.w;
            }
            uint32_t w[4];
#pragma unroll
            for (int i = 0; i < 8; i += 2) {
                float g[2];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int j = j0 + i + q;
                    g[q] = valid ? (d0 * w3f[j] + d1 * w3f[NH + j]) * dgelu(z[i + q]) : 0.f;
                }
                w[i / 2] = pack2(g[0], g[1]);
            }
            *reinterpret_cast<uint4 *>(sm + B_A1 + sw_off(row, j0, TILE)) =
                make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const uint16_t hv = (uint16_t)((w[i / 2] >> ((i & 1) * 16)) & 0xFFFFu);
                *reinterpret_cast<uint16_t *>(sm + B_A2 + sw_off(j0 + i, row, NH)) = hv;
            }
        }
        // h1^T and x^T: column `row`
#pragma unroll 4
        for (int i0 = ch * (NH / 2); i0 < (ch + 1) * (NH / 2); i0 += 8) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (valid) v = __ldg(reinterpret_cast<const uint4 *>(h1s + b * NH + i0));
            const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
                *reinterpret_cast<uint16_t *>(sm + B_H1T + sw_off(i0 + i, row, H1T_ROWS)) =
                    (uint16_t)((wv[i / 2] >> ((i & 1) * 16)) & 0xFFFFu);
        }
#pragma unroll 4
        for (int m0 = ch * (NIN / 2); m0 < (ch + 1) * (NIN / 2); m0 += 8) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (valid) v = __ldg(reinterpret_cast<const uint4 *>(x + b * NIN + m0));
            const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
                *reinterpret_cast<uint16_t *>(sm + B_XT + sw_off(m0 + i, row, XT_ROWS)) =
                    (uint16_t)((wv[i / 2] >> ((i & 1) * 16)) & 0xFFFFu);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            // dh1 [b][i] = dz2 [b][j] W2 [j][i]   (B operand W2^T: rows i, K = j)
#pragma unroll
            for (int s = 0; s < NH / 16; ++s)
                mma_bf16(tbase + T_DH1, sdesc_sw128(sw_kstep(sA1, s, TILE)),
                         sdesc_sw128(sw_kstep(sW2T, s, NH)), idesc_bf16(128, NH), s > 0);
            // dW2 [j][i] (+ db2 at column 128) += dz2^T [j][b] h1 [b][i]
#pragma unroll
            for (int s = 0; s < TILE / 16; ++s)
                mma_bf16(tbase + T_DW2, sdesc_sw128(sw_kstep(sA2, s, NH)),
                         sdesc_sw128(sw_kstep(sH1T, s, H1T_ROWS)), idesc_bf16(128, H1T_ROWS),
                         (s > 0 || !first) ? 1u : 0u);
            mma_commit(bar);
        }
        // this row's half of z1, requested while the tensor cores work
        float z1r[NH / 2];
#pragma unroll
        for (int q = 0; q < NH / 8; ++q) {
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) a = *reinterpret_cast<const float4 *>(z1s + b * NH + ch * (NH / 2) + 4 * q);
            z1r[4 * q] = a.x; z1r[4 * q + 1] = a.y; z1r[4 * q + 2] = a.z; z1r[4 * q + 3] = a.w;
        }
        ok = mbar_wait(bar, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) break;
        tc_fence_after();

        // dz1 = dh1 * gelu'(z1) -> column `row` of A2 (its previous content is consumed)
#pragma unroll
        for (int cc = 0; cc < NH / 32; ++cc) {
            const int c0 = ch * (NH / 2) + 16 * cc;
            float v[16];
            tmem_ld16(tbase + T_DH1 + lane_base + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const float g = valid ? v[i] * dgelu(z1r[16 * cc + i]) : 0.f;
                *reinterpret_cast<__nv_bfloat16 *>(sm + B_A2 + sw_off(c0 + i, row, NH)) =
                    __float2bfloat16_rn(g);
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            // dW1 [j][m] (+ db1 at column 192) += dz1^T [j][b] x [b][m]
#pragma unroll
            for (int s = 0; s < TILE / 16; ++s)
                mma_bf16(tbase + T_DW1, sdesc_sw128(sw_kstep(sA2, s, NH)),
                         sdesc_sw128(sw_kstep(sXT, s, XT_ROWS)), idesc_bf16(128, XT_ROWS),
                         (s > 0 || !first) ? 1u : 0u);
            mma_commit(bar);
        }
        ok = mbar_wait(bar, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) break;
        tc_fence_after();
        first = false;
    }

    if (ok && !first) {
        // row j = `row` of the accumulated weight (and bias) gradients; the
        // two warps of a lane quarter split the 16-column chunks
        float *P = part + (int64_t)blockIdx.x * PART_STRIDE;
        constexpr int C2 = H1T_ROWS / 16, C1 = XT_ROWS / 16;
#pragma unroll 1
        for (int k = ch ? (C2 + 1) / 2 : 0; k < (ch ? C2 : (C2 + 1) / 2); ++k) {
            const int c0 = 16 * k;
            float v[16];
            tmem_ld16(tbase + T_DW2 + lane_base + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int c = c0 + i;
                if (c < NH) P[OFF_W2 + row * NH + c] = v[i];
                else if (c == NH) P[OFF_B2 + row] = v[i];
            }
        }
#pragma unroll 1
        for (int k = ch ? (C1 + 1) / 2 : 0; k < (ch ? C1 : (C1 + 1) / 2); ++k) {
            const int c0 = 16 * k;
            float v[16];
            tmem_ld16(tbase + T_DW1 + lane_base + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int c = c0 + i;
                if (c < NIN) P[OFF_W1 + row * NIN + c] = v[i];
                else if (c == NIN) P[OFF_B1 + row] = v[i];
            }
        }
    } else if (first) {
        float *P = part + (int64_t)blockIdx.x * PART_STRIDE;
        for (int i = t; i < OFF_W3; i += THREADS) P[i] = 0.f;
    }
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if (lane == 0) red[warp] = loss;
    if (!ok && t == 0) atomicOr(err, SPH_EFLAG_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (t == 0) {
        float sum = 0.f;
        for (int w = 0; w < THREADS / 32; ++w) sum += red[w];
        part_loss[blockIdx.x] = 0.5f * inv_count * sum;
    }
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tbase, B_TMEM_COLS);
    }
}

// ---------------------------------------------------------------------------
// backward with TMA tiles and MN-major operands
// ---------------------------------------------------------------------------
// The weight gradients contract over the samples of a tile: dW2 [j][i] =
// sum_b dz2 [b][j] h1 [b][i].  Their operands stay in the sample-major
// layout they arrive in (h1 and x tiles by TMA, dz2 and dz1 written one row
// per thread): read with MN-major descriptors (the contiguous dimension is M
// or N, K = samples strides across 128-byte rows), so nothing is
// transposed.  The same bytes serve as K-major operands where the
// contraction runs along the row (dh1 = dz2 W2 and the recomputed z2 =
// h1 W2^T + b2, which replaces reading the saved z2).  The next tile's h1
// and x are loaded while this tile's epilogues run.
//
// Shared memory, 1024-byte aligned: 14 atoms of 16 KB (128 rows x 128
// bytes, 128-byte swizzling), placed so that every operand's blocks sit at
// one stride (the descriptors' offsets):
//   0 h1 [b][0:64]    1-2 A1 = dz2 [b][j], then A2 = dz1 [b][j]
//   3 W2^T [i][0:64]  4 h1 [b][64:128]     5-7 x [b][m]
//   8 ones (first column 1: the bias gradients db2, db1 in the dW products
//     of h1 and x)    9 W2^T [i][64:128]   10-13 z1 [b][j] in FP32 (32
//                                              columns per atom)
// So h1 as the dW2 operand has blocks 0, 4, 8 (stride 4 atoms), x blocks
// 5 .. 8, W2^T blocks 3, 9.
constexpr uint32_t R_AH1 = 0, R_AA = 1, R_AW2T = 3, R_AX = 5, R_AONE = 8, R_AZ1 = 10,
                   R_ATOMS = 14;
constexpr uint32_t R_B2 = R_ATOMS * ATOM;             // float [128]
constexpr uint32_t R_W3 = R_B2 + NH * 4;              // float [2][128]
constexpr uint32_t R_RED = R_W3 + NOUT * NH * 4;      // float [16] loss per warp
// mbarriers: TMA tiles full (h1, x, z1); products done (z2, dh1, dW2, dW1);
// epilogue steps done (A1 written and z1 read, dh1 read, A2 written)
enum RBar { RB_H = 0, RB_X, RB_Z, RB_FZ, RB_FDH, RB_EH, RB_EX, RB_A1, RB_ZC, RB_A2, RB_N };
constexpr uint32_t R_BAR = R_RED + 16 * 4;
constexpr uint32_t R_SLOT = R_BAR + RB_N * 8;
constexpr uint32_t R_ABORT = R_SLOT + 4;
constexpr uint32_t R_BYTES = R_ABORT + 4 + 1024;      // + alignment of the base
static_assert(R_BYTES <= 232448, "shared memory of one CTA");
constexpr int R_EPI = 16;                             // epilogue warps: four per lane quarter
constexpr int R_THREADS = 32 * (R_EPI + 1);           // + the TMA / MMA warp
constexpr int R_COLS = NH / (R_EPI / 4);              // 32 columns per epilogue warp
// tensor memory: z2, then dh1, at 0 (128 columns); dW2 | db2 at 128 (144);
// dW1 | db1 at 288 (208)
constexpr uint32_t R_TZ = 0, R_TW2 = 128, R_TW1 = 288;
constexpr int R_N2 = NH + 16, R_N1 = NIN + 16;
static_assert(R_TW2 + R_N2 <= R_TW1 && R_TW1 + R_N1 <= 512, "tensor memory plan");
// Shared-memory matrix descriptor, MN-major with 128-byte swizzling: blocks
// of 64 elements along M (or N) at lbo bytes, groups of eight K rows at
// 1024 B (version 1, swizzle mode 2).  A K step of 16 advances the start by
// two groups (2048 B).
__device__ __forceinline__ uint64_t sdesc_sw128_mn(uint32_t saddr, uint32_t lbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// kind::f16 instruction descriptor with MN-major A (bit 15) and / or B (bit 16)
constexpr uint32_t idesc_bf16_mn(int M, int N, bool a_mn, bool b_mn) {
    return idesc_bf16(M, N) | (a_mn ? 1u << 15 : 0u) | (b_mn ? 1u << 16 : 0u);
}

struct BwdMaps {
    CUtensorMap x, h1, z1;
};

// Warp-specialised: warp 16 issues the TMA loads and the products, warps
// 0-15 run the epilogues.  Per tile i (the products in tensor-core order):
//   z2(i) = h1 W2^T              after h1(i) landed and dh1(i-1) was read
//   dW1(i-1) += dz1^T x          after A2(i-1) was written
//   dh1(i) = dz2 W2, dW2(i) += dz2^T h1   after A1(i) was written
// so the tensor cores work on z2(i + 1) and dW1(i) while the epilogue warps
// compute dz1(i), and on dW2(i) during the same epilogue.  h1(i + 1) is
// loaded once dW2(i) has read h1(i), z1(i + 1) once every epilogue warp has
// read z1(i), x(i) once dW1(i - 1) has read x(i - 1).
__global__ void __launch_bounds__(R_THREADS, 1)
    k_mlp_bwd_tma(const __grid_constant__ BwdMaps maps, const MlpDev W,
                  const float *__restrict__ y, const float *__restrict__ target, int64_t n,
                  float inv_count, float *__restrict__ dy_out, float *__restrict__ part,
                  float *__restrict__ part_loss, unsigned *err) {
    extern __shared__ __align__(1024) uint8_t rsm_raw[];
    const uint32_t raw = smem_u32(rsm_raw);
    uint8_t *sm = rsm_raw + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t sbase = smem_u32(sm);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    float *b2f = reinterpret_cast<float *>(sm + R_B2);
    float *w3f = reinterpret_cast<float *>(sm + R_W3);
    float *red = reinterpret_cast<float *>(sm + R_RED);
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + R_SLOT);
    volatile int *abort = reinterpret_cast<volatile int *>(sm + R_ABORT);
    auto bar = [&](int i) { return sbase + R_BAR + 8u * (uint32_t)i; };
    auto atom = [&](uint32_t k) { return sbase + k * ATOM; };

    // W2^T [i][j] into atoms 3 and 9 (columns j 0-63, 64-127)
    for (int c = t; c < NH * (NH / 8); c += R_THREADS) {
        const int r = c >> 4, k8 = c & 15;
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(W.w2t + r * NH + k8 * 8));
        const uint32_t a = k8 < 8 ? R_AW2T : R_AW2T + 6;
        *reinterpret_cast<uint4 *>(sm + a * ATOM + sw128_off(r, k8 & 7)) = v;
    }
    for (int i = t; i < NH; i += R_THREADS) b2f[i] = W.params[OFF_B2 + i];
    for (int i = t; i < NOUT * NH; i += R_THREADS) w3f[i] = __uint_as_float((uint32_t)W.w3[i] << 16);
    // the ones atom: column 0 one, the rest zero
    for (int c = t; c < TILE * 8; c += R_THREADS) {
        const int r = c >> 3, k = c & 7;
        *reinterpret_cast<uint4 *>(sm + R_AONE * ATOM + sw128_off(r, k)) =
            make_uint4(k == 0 ? 0x3F80u : 0u, 0u, 0u, 0u);
    }
    if (t == 0) {
        *abort = 0;
        for (int k = 0; k < RB_N; ++k)
            mbar_init(bar(k), (k == RB_A1 || k == RB_ZC || k == RB_A2) ? R_EPI : 1);
    }
    if (warp == 0) tmem_alloc(smem_u32(slot), 512);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *slot;
    const int64_t ntiles = (n + TILE - 1) / TILE;
    const int mine = ntiles > blockIdx.x ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    auto tile_row0 = [&](int i) { return (int)((blockIdx.x + (int64_t)i * gridDim.x) * TILE); };
    bool ok = true;

    if (warp == R_EPI) {
        if (lane == 0) {
            // ---- TMA loads and products ----
            auto load_h1 = [&](int i) {
                mbar_expect_tx(bar(RB_H), 2 * ATOM);
                tma_load_2d(atom(R_AH1), &maps.h1, bar(RB_H), 0, tile_row0(i));
                tma_load_2d(atom(R_AH1 + 4), &maps.h1, bar(RB_H), 64, tile_row0(i));
            };
            auto load_x = [&](int i) {
                mbar_expect_tx(bar(RB_X), 3 * ATOM);
                for (int a = 0; a < 3; ++a)
                    tma_load_2d(atom(R_AX + a), &maps.x, bar(RB_X), 64 * a, tile_row0(i));
            };
            auto load_z1 = [&](int i) {
                mbar_expect_tx(bar(RB_Z), 4 * ATOM);
                for (int a = 0; a < 4; ++a)
                    tma_load_2d(atom(R_AZ1 + a), &maps.z1, bar(RB_Z), 32 * a, tile_row0(i));
            };
            // K step s (16 of 128) of a K-major operand in atoms a0 (K 0-63) and a1
            auto kstep = [&](uint32_t a0, uint32_t a1, int s) {
                return atom(s < 4 ? a0 : a1) + (uint32_t)(s & 3) * 32;
            };
            constexpr uint32_t ID_Z = idesc_bf16_mn(128, NH, false, true);
            constexpr uint32_t ID_DH = idesc_bf16(128, NH);
            constexpr uint32_t ID_W2 = idesc_bf16_mn(128, R_N2, true, true);
            constexpr uint32_t ID_W1 = idesc_bf16_mn(128, R_N1, true, true);
            auto dw1 = [&](int i) -> bool {
                // dW1 [j][m] (+ db1 at column 192) += dz1^T [j][b] x [b][m]
                if (!gwait(bar(RB_A2), i & 1, abort) || !gwait(bar(RB_X), i & 1, abort))
                    return false;
                tc_fence_after();
#pragma unroll
                for (int s = 0; s < TILE / 16; ++s)
                    mma_bf16(tbase + R_TW1, sdesc_sw128_mn(atom(R_AA) + 2048u * s, ATOM),
                             sdesc_sw128_mn(atom(R_AX) + 2048u * s, ATOM), ID_W1,
                             (s > 0 || i > 0) ? 1u : 0u);
                mma_commit(bar(RB_EX));
                return true;
            };
            int nh = 0, nx = 0, nz = 0;   // loads issued
            if (mine > 0) {
                load_h1(0);
                load_x(0);
                load_z1(0);
                nh = nx = nz = 1;
            }
            for (int i = 0; i < mine; ++i) {
                // z2(i) = h1 W2^T (the bias added by the epilogue)
                if (!gwait(bar(RB_H), i & 1, abort)) break;
                if (i > 0 && !gwait(bar(RB_ZC), (i - 1) & 1, abort)) break;
                tc_fence_after();
#pragma unroll
                for (int s = 0; s < NH / 16; ++s)
                    mma_bf16(tbase + R_TZ, sdesc_sw128(kstep(R_AH1, R_AH1 + 4, s)),
                             sdesc_sw128_mn(atom(R_AW2T) + 2048u * s, 6 * ATOM), ID_Z, s > 0);
                mma_commit(bar(RB_FZ));
                if (i > 0) {
                    if (!dw1(i - 1)) break;
                    // x(i) once dW1(i - 1) has read x(i - 1)
                    if (!gwait(bar(RB_EX), (i - 1) & 1, abort)) break;
                    load_x(i);
                    ++nx;
                }
                // A1(i) written and z1(i) read: the next z1, then dh1 and dW2
                if (!gwait(bar(RB_A1), i & 1, abort)) break;
                if (i + 1 < mine) {
                    load_z1(i + 1);
                    ++nz;
                }
                tc_fence_after();
                // dh1 [b][i] = dz2 [b][j] W2 [j][i]   (B: W2^T rows i, K = j)
#pragma unroll
                for (int s = 0; s < NH / 16; ++s)
                    mma_bf16(tbase + R_TZ, sdesc_sw128(kstep(R_AA, R_AA + 1, s)),
                             sdesc_sw128(kstep(R_AW2T, R_AW2T + 6, s)), ID_DH, s > 0);
                mma_commit(bar(RB_FDH));
                // dW2 [j][i] (+ db2 at column 128) += dz2^T [j][b] h1 [b][i]
#pragma unroll
                for (int s = 0; s < TILE / 16; ++s)
                    mma_bf16(tbase + R_TW2, sdesc_sw128_mn(atom(R_AA) + 2048u * s, ATOM),
                             sdesc_sw128_mn(atom(R_AH1) + 2048u * s, 4 * ATOM), ID_W2,
                             (s > 0 || i > 0) ? 1u : 0u);
                mma_commit(bar(RB_EH));
                // h1(i + 1) once dW2(i) has read h1(i)
                if (i + 1 < mine) {
                    if (!gwait(bar(RB_EH), i & 1, abort)) break;
                    load_h1(i + 1);
                    ++nh;
                }
            }
            if (!*abort && mine > 0 && dw1(mine - 1)) gwait(bar(RB_EX), (mine - 1) & 1, abort);
            // every load issued has landed before the CTA may exit (each
            // barrier has at most its last phase outstanding; a bounded wait
            // that does not give up on the abort word)
            if (nh > 0) mbar_wait(bar(RB_H), (nh - 1) & 1);
            if (nx > 0) mbar_wait(bar(RB_X), (nx - 1) & 1);
            if (nz > 0) mbar_wait(bar(RB_Z), (nz - 1) & 1);
        }
        __syncwarp();
    } else {
        // ---- epilogues: row = sample (tensor-memory lane), 32 columns ----
        const int q = warp & 3, cp = warp >> 2;
        const int row = q * 32 + lane;
        const int cb = cp * R_COLS;
        const uint32_t lane_base = (uint32_t)(q * 32) << 16;
        float loss = 0.f;
        float4 yt = make_float4(0.f, 0.f, 0.f, 0.f);
        auto load_yt = [&](int i) {
            const int64_t b = (int64_t)tile_row0(i) + row;
            if (b < n) {
                const float2 a = *reinterpret_cast<const float2 *>(y + b * 2);
                const float2 c = *reinterpret_cast<const float2 *>(target + b * 2);
                yt = make_float4(a.x, a.y, c.x, c.y);
            }
        };
        auto store_rows = [&](uint32_t base_atom, int c, const uint32_t (&w)[8]) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int col = cb + 16 * c + 8 * k;
                *reinterpret_cast<uint4 *>(sm + (base_atom + (col >> 6)) * ATOM +
                                           sw128_off(row, (col & 63) >> 3)) =
                    make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
            }
        };
        // a wait every lane of the warp agrees on (the tensor-memory loads
        // after it are warp-wide)
        auto wwait = [&](int k, int parity) {
            return __all_sync(0xffffffffu, gwait(bar(k), (uint32_t)parity & 1u, abort)) != 0;
        };
        if (mine > 0) load_yt(0);
        for (int i = 0; i < mine; ++i) {
            const int64_t b = (int64_t)tile_row0(i) + row;
            const bool valid = b < n;
            float d0 = 0.f, d1 = 0.f;
            if (valid) {
                const float e0 = yt.x - yt.z, e1 = yt.y - yt.w;
                d0 = e0 * inv_count;
                d1 = e1 * inv_count;
                if (cp == 0) {
                    loss += e0 * e0 + e1 * e1;
                    *reinterpret_cast<float2 *>(dy_out + b * 2) = make_float2(d0, d1);
                }
            }
            if (i + 1 < mine) load_yt(i + 1);
            // dz2 = (dy W3) * gelu'(z2 + b2), written once dW1(i - 1) has
            // read A2(i - 1) (the same atoms)
            if (!wwait(RB_FZ, i)) { ok = false; break; }
            tc_fence_after();
            uint32_t w2[2][8];
            const uint64_t dd0 = valid ? f2(d0, d0) : f2(0.f, 0.f);
            const uint64_t dd1 = valid ? f2(d1, d1) : f2(0.f, 0.f);
            uint32_t rz[2][16];
            tmem_ld16_async(tbase + R_TZ + lane_base + cb, rz[0]);
            tmem_wait16(rz[0]);
            tmem_ld16_async(tbase + R_TZ + lane_base + cb + 16, rz[1]);
#pragma unroll
            for (int c = 0; c < R_COLS / 16; ++c) {
                if (c == 1) tmem_wait16(rz[1]);
                float v[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) v[e] = __uint_as_float(rz[c][e]);
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    // columns j, j + 1, two per packed instruction
                    const int j = cb + 16 * c + 2 * e;
                    const uint64_t z = add2(f2(v[2 * e], v[2 * e + 1]),
                                            *reinterpret_cast<const uint64_t *>(b2f + j));
                    const uint64_t g = fma2(dd1, *reinterpret_cast<const uint64_t *>(w3f + NH + j),
                                            mul2(dd0, *reinterpret_cast<const uint64_t *>(w3f + j)));
                    float g0, g1;
                    f2_split(mul2(g, dgelu2(z)), g0, g1);
                    w2[c][e] = pack2(g0, g1);
                }
            }
            if (i > 0 && !wwait(RB_EX, i - 1)) { ok = false; break; }
#pragma unroll
            for (int c = 0; c < R_COLS / 16; ++c) store_rows(R_AA, c, w2[c]);
            // this row's z1 columns cb .. cb + 31: atom cb / 32 of the z1 tile
            if (!wwait(RB_Z, i)) { ok = false; break; }
            float z1r[R_COLS];
#pragma unroll
            for (int k = 0; k < R_COLS / 4; ++k) {
                const float4 a = *reinterpret_cast<const float4 *>(sm + (R_AZ1 + cp) * ATOM + sw128_off(row, k));
                z1r[4 * k] = a.x; z1r[4 * k + 1] = a.y; z1r[4 * k + 2] = a.z; z1r[4 * k + 3] = a.w;
            }
            fence_async_smem();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(RB_A1));
            // dz1 = dh1 * gelu'(z1) -> A2, once dW2(i) has read A1(i)
            if (!wwait(RB_FDH, i)) { ok = false; break; }
            tc_fence_after();
            float v[R_COLS];
            {
                uint32_t rh[2][16];
                tmem_ld16_async(tbase + R_TZ + lane_base + cb, rh[0]);
                tmem_ld16_async(tbase + R_TZ + lane_base + cb + 16, rh[1]);
                tmem_wait16(rh[0]);
                tmem_wait16(rh[1]);
#pragma unroll
                for (int c = 0; c < 2; ++c)
#pragma unroll
                    for (int e = 0; e < 16; ++e) v[16 * c + e] = __uint_as_float(rh[c][e]);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(RB_ZC));
            uint32_t w1[2][8];
#pragma unroll
            for (int c = 0; c < R_COLS / 16; ++c) {
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int k = 16 * c + 2 * e;
                    float g0, g1;
                    f2_split(mul2(f2(v[k], v[k + 1]), dgelu2(f2(z1r[k], z1r[k + 1]))), g0, g1);
                    w1[c][e] = valid ? pack2(g0, g1) : 0u;
                }
            }
            if (!wwait(RB_EH, i)) { ok = false; break; }
#pragma unroll
            for (int c = 0; c < R_COLS / 16; ++c) store_rows(R_AA, c, w1[c]);
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(RB_A2));
        }
        // every product has finished before the gradients are read
        if (ok && mine > 0 && !wwait(RB_EX, mine - 1)) ok = false;
        for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
        if (lane == 0) red[warp] = loss;
        tc_fence_after();
        float *P = part + (int64_t)blockIdx.x * PART_STRIDE;
        if (ok && !*abort && mine > 0) {
            // row j = `row` of the accumulated weight (and bias) gradients; the
            // four warps of a lane quarter take every fourth 16-column chunk
#pragma unroll 1
            for (int k = cp; k < R_N2 / 16; k += 4) {
                const int c0 = 16 * k;
                float u[16];
                tmem_ld16(tbase + R_TW2 + lane_base + c0, u);
                if (c0 < NH) {
                    float4 *dst = reinterpret_cast<float4 *>(P + OFF_W2 + row * NH + c0);
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        dst[e] = make_float4(u[4 * e], u[4 * e + 1], u[4 * e + 2], u[4 * e + 3]);
                } else {
                    P[OFF_B2 + row] = u[0];
                }
            }
#pragma unroll 1
            for (int k = cp; k < R_N1 / 16; k += 4) {
                const int c0 = 16 * k;
                float u[16];
                tmem_ld16(tbase + R_TW1 + lane_base + c0, u);
                if (c0 < NIN) {
                    float4 *dst = reinterpret_cast<float4 *>(P + OFF_W1 + row * NIN + c0);
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        dst[e] = make_float4(u[4 * e], u[4 * e + 1], u[4 * e + 2], u[4 * e + 3]);
                } else {
                    P[OFF_B1 + row] = u[0];
                }
            }
        } else if (mine == 0) {
            for (int k = t; k < OFF_W3; k += 32 * R_EPI) P[k] = 0.f;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (t == 0) {
        if (*abort || !ok) atomicOr(err, SPH_EFLAG_TIMEOUT);
        float sum = 0.f;
        for (int w = 0; w < R_EPI; ++w) sum += red[w];
        part_loss[blockIdx.x] = 0.5f * inv_count * sum;
    }
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tbase, 512);
    }
}

// third layer: dW3 [o][j] = sum_b dy[b][o] h2[b][j], db3 = sum_b dy
__global__ void k_mlp_l3(const uint16_t *__restrict__ h2s, const float *__restrict__ dy,
                         int64_t n, float *__restrict__ part) {
    const int j = threadIdx.x;   // 128 threads
    const int64_t r0 = (int64_t)blockIdx.x * L3_ROWS;
    const int64_t r1 = min(n, r0 + L3_ROWS);
    float a0 = 0.f, a1 = 0.f, s0 = 0.f, s1 = 0.f;
    for (int64_t b = r0; b < r1; ++b) {
        const float h = __uint_as_float((uint32_t)h2s[b * NH + j] << 16);
        const float d0 = dy[b * 2], d1 = dy[b * 2 + 1];
        a0 = fmaf(d0, h, a0);
        a1 = fmaf(d1, h, a1);
        s0 += d0;
        s1 += d1;
    }
    float *P = part + (int64_t)blockIdx.x * L3_PART;
    P[j] = a0;
    P[NH + j] = a1;
    if (j == 0) {
        P[2 * NH] = s0;
        P[2 * NH + 1] = s1;
    }
}

// grad[p] = sum over CTAs (fixed order) of the partials
__global__ void k_mlp_reduce(const float *__restrict__ part, int nparts,
                             const float *__restrict__ l3, int nl3,
                             const float *__restrict__ part_loss, float *__restrict__ grad,
                             float *__restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < OFF_W3) {
        float s = 0.f;
        for (int c = 0; c < nparts; ++c) s += part[(int64_t)c * PART_STRIDE + p];
        grad[p] = s;
    } else if (p < NPARAM) {
        float s = 0.f;
        for (int c = 0; c < nl3; ++c) s += l3[(int64_t)c * L3_PART + (p - OFF_W3)];
        grad[p] = s;
    } else if (p == NPARAM && loss) {
        float s = 0.f;
        for (int c = 0; c < nparts; ++c) s += part_loss[c];
        *loss = s;
    }
}

__device__ __forceinline__ void write_copies(const MlpDev &W, uint16_t *w1, uint16_t *w2,
                                             uint16_t *w2t, uint16_t *w3, int p, float v) {
    const uint16_t b = __bfloat16_as_ushort(__float2bfloat16_rn(v));
    if (p < OFF_B1) {
        w1[p] = b;
    } else if (p >= OFF_W2 && p < OFF_B2) {
        const int q = p - OFF_W2, r = q / NH, c = q % NH;
        w2[q] = b;
        w2t[c * NH + r] = b;
    } else if (p >= OFF_W3 && p < OFF_B3) {
        w3[p - OFF_W3] = b;
    }
}

__global__ void k_mlp_sync(const float *__restrict__ params, uint16_t *w1, uint16_t *w2,
                           uint16_t *w2t, uint16_t *w3) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < NPARAM) write_copies(MlpDev{}, w1, w2, w2t, w3, p, params[p]);
}

__global__ void k_mlp_adam(float *__restrict__ params, const float *__restrict__ grad,
                           float *__restrict__ m, float *__restrict__ v, float lr, float beta1,
                           float beta2, float eps, float c1, float c2, uint16_t *w1,
                           uint16_t *w2, uint16_t *w2t, uint16_t *w3) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    const float g = grad[p];
    const float mp = beta1 * m[p] + (1.f - beta1) * g;
    const float vp = beta2 * v[p] + (1.f - beta2) * g * g;
    m[p] = mp;
    v[p] = vp;
    const float val = params[p] - lr * (mp * c1) / (sqrtf(vp * c2) + eps);
    params[p] = val;
    write_copies(MlpDev{}, w1, w2, w2t, w3, p, val);
}

// acc[c][i] (+)= (y[i][c] * scale[c] + mean[c]) * c0^2 / h_i for real particles
__global__ void k_mlp_apply(int64_t n, const float *__restrict__ yv, const int64_t *__restrict__ tag,
                            const double *__restrict__ h, double c0sq, double s0, double s1,
                            double m0, double m1, double *ax, double *ay, double *az,
                            int accumulate) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool real = tag == nullptr || tag[i] == SPH_TAG_LOCAL_REAL;
    // in FP32 (the network's output carries BF16-level error): an FP64
    // division costs a warp about ten instructions on GB300's narrow FP64
    // pipe, and this kernel did little else
    const float f = real ? __fdiv_rn((float)c0sq, (float)h[i]) : 0.f;
    const double a0 = real ? (double)(fmaf(yv[2 * i], (float)s0, (float)m0) * f) : 0.0;
    const double a1 = real ? (double)(fmaf(yv[2 * i + 1], (float)s1, (float)m1) * f) : 0.0;
    if (accumulate) {
        if (ax) ax[i] += a0;
        if (ay) ay[i] += a1;
    } else {
        if (ax) ax[i] = a0;
        if (ay) ay[i] = a1;
        if (az) az[i] = 0.0;
    }
}

// out[i] = ((a[i] * h_i / c0^2) - mean) * inv_std, two components
__global__ void k_mlp_targets(int64_t n, const double *__restrict__ ax, const double *__restrict__ ay,
                              const double *__restrict__ h, double inv_c0sq, double m0, double m1,
                              double is0, double is1, float *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double f = h[i] * inv_c0sq;
    out[2 * i] = (float)((ax[i] * f - m0) * is0);
    out[2 * i + 1] = (float)((ay[i] * f - m1) * is1);
}

int g_num_sms = 0;
std::once_flag g_attr_once;
cudaError_t g_attr_err = cudaSuccess;

// the driver's tensor-map encoder, through the runtime's entry-point lookup
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                 const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                 const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled g_encode = nullptr;

cudaError_t init_attrs() {
    std::call_once(g_attr_once, [] {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, F_BYTES);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_mlp_fwd_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     G_BYTES);
        if (e == cudaSuccess) {
            void *fn = nullptr;
            cudaDriverEntryPointQueryResult q;
            e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                 cudaEnableDefault, &q);
            if (e == cudaSuccess && q == cudaDriverEntryPointSuccess)
                g_encode = reinterpret_cast<EncodeTiled>(fn);
        }
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_mlp_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, B_BYTES);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_mlp_bwd_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     R_BYTES);
        g_attr_err = e;
    });
    return g_attr_err;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// Tensor map of a row-major BF16 matrix [rows][cols] (cols a multiple of
// 64): boxes of 64 columns x 128 rows with 128-byte swizzling; rows past
// the end read as zeros.
int encode_rows(CUtensorMap *m, const void *base, uint64_t rows, uint64_t cols) {
    if (!g_encode) return set_error(SPH_ERR_CUDA, "mlp: the tensor-map encoder is unavailable");
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 2};
    const cuuint32_t box[2] = {64, 128};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims,
                                strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(SPH_ERR_CUDA, "mlp: cuTensorMapEncodeTiled failed");
    return SPH_OK;
}

// Tensor map of a row-major FP32 matrix [rows][cols] (cols a multiple of
// 32): boxes of 32 columns (128 bytes) x 128 rows with 128-byte swizzling.
int encode_rows_f32(CUtensorMap *m, const void *base, uint64_t rows, uint64_t cols) {
    if (!g_encode) return set_error(SPH_ERR_CUDA, "mlp: the tensor-map encoder is unavailable");
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 4};
    const cuuint32_t box[2] = {32, 128};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base), dims,
                                strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(SPH_ERR_CUDA, "mlp: cuTensorMapEncodeTiled failed");
    return SPH_OK;
}

// environment SPH_MLP_FWD_LEGACY=1: the forward kernel without TMA and
// warp specialisation, to measure against
bool legacy_forward() {
    static int v = -1;
    if (v < 0) {
        const char *e = getenv("SPH_MLP_FWD_LEGACY");
        v = (e && atoi(e) > 0) ? 1 : 0;
    }
    return v == 1;
}

// environment SPH_MLP_BWD_LEGACY=1: the backward kernel that stages
// transposed copies of its operands and reads the saved z2
bool legacy_backward() {
    static int v = -1;
    if (v < 0) {
        const char *e = getenv("SPH_MLP_BWD_LEGACY");
        v = (e && atoi(e) > 0) ? 1 : 0;
    }
    return v == 1;
}

}  // namespace

int mlp_grid(int64_t n) {
    if (init_attrs() != cudaSuccess) return 0;
    const int64_t tiles = (n + TILE - 1) / TILE;
    return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, g_num_sms));
}

int64_t mlp_backward_scratch(int64_t n) {
    const int grid = mlp_grid(n);
    const int64_t nl3 = (n + L3_ROWS - 1) / L3_ROWS;
    return (int64_t)grid * PART_STRIDE + std::max<int64_t>(nl3, 1) * L3_PART + grid + 2 * n + 4;
}

int mlp_sync(const sph_mlp_model *M, cudaStream_t st) {
    k_mlp_sync<<<(NPARAM + 255) / 256, 256, 0, st>>>(M->params, M->w1, M->w2, M->w2t, M->w3);
    count_launch();
    SPH_LAUNCH_CHECK("k_mlp_sync");
    return SPH_OK;
}

int mlp_forward(const sph_mlp_model *M, const uint16_t *x, int64_t n, float *y, float *z1,
                float *z2, uint16_t *h1, uint16_t *h2, unsigned *err, cudaStream_t st) {
    if (n <= 0) return SPH_OK;
    if (!aligned16(x) || (z1 && !aligned16(z1)) || (z2 && !aligned16(z2)) || (h1 && !aligned16(h1)) ||
        (h2 && !aligned16(h2)) || !aligned16(M->w1) || !aligned16(M->w2))
        return set_error(SPH_ERR_ARG, "mlp forward: buffers must be 16-byte aligned");
    SPH_CUDA(init_attrs());
    if (legacy_forward()) {
        const MlpDev W{M->params, M->w1, M->w2, M->w2t, M->w3};
        k_mlp_fwd<<<mlp_grid(n), THREADS, F_BYTES, st>>>(W, x, n, y, z1, z2, h1, h2, err);
        count_launch();
        SPH_LAUNCH_CHECK("k_mlp_fwd");
        return SPH_OK;
    }
    MlpMaps maps;
    int rc = encode_rows(&maps.x, x, (uint64_t)n, NIN);
    if (!rc) rc = encode_rows(&maps.w1, M->w1, NH, NIN);
    if (!rc) rc = encode_rows(&maps.w2, M->w2, NH, NH);
    if (rc) return rc;
    k_mlp_fwd_tma<<<mlp_grid(n), G_THREADS, G_BYTES, st>>>(maps, M->params, M->w3, n, y, z1, z2,
                                                             h1, h2, err);
    count_launch();
    SPH_LAUNCH_CHECK("k_mlp_fwd_tma");
    return SPH_OK;
}

int mlp_backward(const sph_mlp_model *M, const uint16_t *x, const uint16_t *h1, const uint16_t *h2,
                 const float *z1, const float *z2, const float *y, const float *target, int64_t n,
                 float inv_count, float *grad, float *loss, float *scratch, unsigned *err,
                 cudaStream_t st) {
    if (n <= 0) return set_error(SPH_ERR_ARG, "mlp backward: empty batch");
    if (!aligned16(x) || !aligned16(h1) || !aligned16(z1) || !aligned16(z2) || !aligned16(M->w2t))
        return set_error(SPH_ERR_ARG, "mlp backward: buffers must be 16-byte aligned");
    SPH_CUDA(init_attrs());
    const int grid = mlp_grid(n);
    const int nl3 = (int)std::max<int64_t>(1, (n + L3_ROWS - 1) / L3_ROWS);
    float *part = scratch;
    float *l3 = part + (int64_t)grid * PART_STRIDE;
    float *part_loss = l3 + (int64_t)nl3 * L3_PART;
    float *dy = part_loss + grid;
    dy = reinterpret_cast<float *>(((uintptr_t)dy + 15) & ~(uintptr_t)15);
    const MlpDev W{M->params, M->w1, M->w2, M->w2t, M->w3};
    if (legacy_backward()) {
        k_mlp_bwd<<<grid, THREADS, B_BYTES, st>>>(W, x, h1, z1, z2, y, target, n, inv_count, dy,
                                                   part, part_loss, err);
        count_launch();
        SPH_LAUNCH_CHECK("k_mlp_bwd");
    } else {
        BwdMaps maps;
        int rc = encode_rows(&maps.x, x, (uint64_t)n, NIN);
        if (!rc) rc = encode_rows(&maps.h1, h1, (uint64_t)n, NH);
        if (!rc) rc = encode_rows_f32(&maps.z1, z1, (uint64_t)n, NH);
        if (rc) return rc;
        k_mlp_bwd_tma<<<grid, R_THREADS, R_BYTES, st>>>(maps, W, y, target, n, inv_count, dy, part,
                                                         part_loss, err);
        count_launch();
        SPH_LAUNCH_CHECK("k_mlp_bwd_tma");
    }
    k_mlp_l3<<<nl3, NH, 0, st>>>(h2, dy, n, l3);
    count_launch();
    SPH_LAUNCH_CHECK("k_mlp_l3");
    k_mlp_reduce<<<(NPARAM + 1 + 255) / 256, 256, 0, st>>>(part, grid, l3, nl3, part_loss, grad, loss);
    count_launch();
    SPH_LAUNCH_CHECK("k_mlp_reduce");
    return SPH_OK;
}

int mlp_adam(const sph_mlp_model *M, const float *grad, float *m, float *v, float lr, float beta1,
             float beta2, float eps, int step, cudaStream_t st) {
    if (step < 1) return set_error(SPH_ERR_ARG, "mlp adam: step counts from 1");
    const float c1 = (float)(1.0 / (1.0 - std::pow((double)beta1, step)));
    const float c2 = (float)(1.0 / (1.0 - std::pow((double)beta2, step)));
    k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, st>>>(M->params, grad, m, v, lr, beta1, beta2, eps,
                                                      c1, c2, M->w1, M->w2, M->w2t, M->w3);
    count_launch();
    SPH_LAUNCH_CHECK("k_mlp_adam");
    return SPH_OK;
}

int mlp_apply(int64_t n, const float *y, const int64_t *tag, const double *h, double c0,
              const double *scale, const double *mean, double *const *acc, int accumulate,
              cudaStream_t st) {
    if (n <= 0) return SPH_OK;
    k_mlp_apply<<<(int)((n + 255) / 256), 256, 0, st>>>(n, y, tag, h, c0 * c0, scale[0], scale[1],
                                                        mean[0], mean[1], acc[0], acc[1], acc[2],
                                                        accumulate);
    count_launch();
    SPH_LAUNCH_CHECK("k_mlp_apply");
    return SPH_OK;
}

int mlp_targets(int64_t n, const double *ax, const double *ay, const double *h, double c0,
                const double *mean, const double *inv_std, float *out, cudaStream_t st) {
    if (n <= 0) return SPH_OK;
    k_mlp_targets<<<(int)((n + 255) / 256), 256, 0, st>>>(n, ax, ay, h, 1.0 / (c0 * c0), mean[0],
                                                          mean[1], inv_std[0], inv_std[1], out);
    count_launch();
    SPH_LAUNCH_CHECK("k_mlp_targets");
    return SPH_OK;
}

}  // namespace sphgb
