// C ABI of the pysph_gb300 library: context management, argument checks and
// error reporting around the kernels of nnps.cu, pairs.cu and elementwise.cu.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <new>
#include <string>

#include "sph_internal.cuh"

namespace sphgb {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int set_error(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int cuda_check(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return SPH_ERR_CUDA;
}

int red_part_doubles();

namespace {

__global__ void k_sum_i64(const int64_t *v, int64_t n, unsigned long long *out) {
    unsigned long long s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        s += (unsigned long long)v[i];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

}  // namespace

}  // namespace sphgb

using namespace sphgb;

#define CHECK_CTX(c)                                                     \
    do {                                                                 \
        if (!(c)) return set_error(SPH_ERR_ARG, "null sph_ctx");         \
    } while (0)

extern "C" {

int sph_version(void) { return 1; }

int sph_launch_count(int64_t *out) {
    if (!out) return set_error(SPH_ERR_ARG, "sph_launch_count: null out");
    *out = (int64_t)g_launches.load(std::memory_order_relaxed);
    return SPH_OK;
}

int sph_last_error(char *buf, size_t len) {
    if (!buf || len == 0) return SPH_ERR_ARG;
    size_t n = g_last_error.size() < len - 1 ? g_last_error.size() : len - 1;
    memcpy(buf, g_last_error.data(), n);
    buf[n] = 0;
    return SPH_OK;
}

int sph_ctx_create(int dim, sph_ctx **out) {
    if (!out) return set_error(SPH_ERR_ARG, "sph_ctx_create: null out");
    if (dim < 1 || dim > 3) return set_error(SPH_ERR_ARG, "sph_ctx_create: dim must be 1..3");
    sph_ctx *c = new (std::nothrow) sph_ctx();
    if (!c) return set_error(SPH_ERR_ARG, "sph_ctx_create: out of host memory");
    c->dim = dim;
    cudaError_t e;
    if ((e = cudaMalloc(&c->d_box, 8 * sizeof(int))) != cudaSuccess ||
        (e = cudaMalloc(&c->d_hmax, 2 * sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMalloc(&c->d_status, kStatusWords * sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMalloc(&c->d_part, sizeof(double) * red_part_doubles())) != cudaSuccess ||
        (e = cudaHostAlloc(&c->h_box, 16 * sizeof(int), cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaMallocHost(&c->h_red, 16 * sizeof(double))) != cudaSuccess ||
        (e = cudaHostAlloc(&c->h_status, kStatusWords * sizeof(unsigned), cudaHostAllocMapped)) !=
            cudaSuccess ||
        (e = cudaHostGetDevicePointer((void **)&c->hd_box, c->h_box, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer((void **)&c->hd_status, c->h_status, 0)) != cudaSuccess ||
        (e = cudaMalloc(&c->d_bstats, 2 * kMaxBrickArrays * sizeof(unsigned))) != cudaSuccess ||
        (e = cudaHostAlloc(&c->h_bstats, 2 * kMaxBrickArrays * sizeof(unsigned),
                           cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer((void **)&c->hd_bstats, c->h_bstats, 0)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&c->pending_event, cudaEventDisableTiming)) != cudaSuccess) {
        sph_ctx_destroy(c);
        return cuda_check(e, "sph_ctx_create");
    }
    cudaMemset(c->d_status, 0, kStatusWords * sizeof(unsigned));
    c->d_err = c->d_status;
    *out = c;
    return SPH_OK;
}

int sph_ctx_destroy(sph_ctx *c) {
    if (!c) return SPH_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_lists(c);
    for (auto &A : c->arrays) {
        cudaFree(A.key); cudaFree(A.perm); cudaFree(A.skey);
        cudaFree(A.scx); cudaFree(A.pm); cudaFree(A.velh); cudaFree(A.st);
        cudaFree(A.nrm); cudaFree(A.tan);
        cudaFree(A.cstart); cudaFree(A.cursor); cudaFree(A.refcell); cudaFree(A.pm0); cudaFree(A.inv);
        cudaFree(A.bdst);
    }
    cudaFree(c->d_box); cudaFree(c->d_hmax); cudaFree(c->d_status);
    cudaFree(c->scan_tmp); cudaFree(c->d_part); cudaFree(c->d_cnt);
    if (c->h_box) cudaFreeHost(c->h_box);
    if (c->h_red) cudaFreeHost(c->h_red);
    if (c->h_status) cudaFreeHost(c->h_status);
    cudaFree(c->d_bstats);
    if (c->h_bstats) cudaFreeHost(c->h_bstats);
    if (c->pending_event) cudaEventDestroy(c->pending_event);
    delete c;
    return SPH_OK;
}

int sph_ctx_set_stream(sph_ctx *c, void *stream) {
    CHECK_CTX(c);
    // a gated pass must follow its refresh on the same stream
    if (c->pending && (cudaStream_t)stream != c->stream) {
        const int rc = resolve_pending(c);
        if (rc) return rc;
    }
    c->stream = (cudaStream_t)stream;
    return SPH_OK;
}

// Entry points that use the neighbour structure (or move particles) read a
// pending deferred refresh first.
#define RESOLVE(c)                              \
    do {                                        \
        const int rc_ = resolve_pending(c);     \
        if (rc_) return rc_;                    \
    } while (0)

// While a step program records (sph_step_begin), the calls a step is made
// of are recorded instead of run; the others are refused.
#define NOT_RECORDING(c, name)                                                          \
    do {                                                                                \
        if ((c)->recording)                                                             \
            return set_error(SPH_ERR_STATE, name ": not recordable in a step program"); \
    } while (0)

int sph_nnps_build(sph_ctx *c, const sph_array_view *arrays, int narrays, double cell_size,
                   double radius_scale, int subdiv, int check_jump) {
    CHECK_CTX(c);
    if (c->recording)
        return record_update(c, true, arrays, narrays, cell_size, radius_scale, subdiv, check_jump);
    RESOLVE(c);
    return nnps_build(c, arrays, narrays, cell_size, radius_scale, subdiv, check_jump);
}

int sph_nnps_update(sph_ctx *c, const sph_array_view *arrays, int narrays, double cell_size,
                    double radius_scale, int subdiv, int check_jump, int *rebuilt) {
    CHECK_CTX(c);
    if (c->recording) {
        if (rebuilt) *rebuilt = 0;
        return record_update(c, false, arrays, narrays, cell_size, radius_scale, subdiv, check_jump);
    }
    return nnps_update(c, arrays, narrays, cell_size, radius_scale, subdiv, check_jump, rebuilt);
}

int sph_ctx_set_deferred(sph_ctx *c, int on) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_ctx_set_deferred");
    if (on != 0 && on != 1) return set_error(SPH_ERR_ARG, "sph_ctx_set_deferred: on must be 0 or 1");
    RESOLVE(c);
    c->deferred = on;
    return SPH_OK;
}

int sph_ctx_set_skin(sph_ctx *c, double skin_fraction) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_ctx_set_skin");
    RESOLVE(c);
    if (!(skin_fraction >= 0.0) || skin_fraction > 0.5)
        return set_error(SPH_ERR_ARG, "sph_ctx_set_skin: fraction must be in [0, 0.5]");
    if (skin_fraction != c->skin_frac) {
        c->skin_frac = skin_fraction;
        c->built = false;   // the next update builds afresh
    }
    return SPH_OK;
}

int sph_ctx_set_symmetric(sph_ctx *c, int on) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_ctx_set_symmetric");
    RESOLVE(c);
    if (on != 0 && on != 1) return set_error(SPH_ERR_ARG, "sph_ctx_set_symmetric: on must be 0 or 1");
    if (on != c->symmetric) {
        c->symmetric = on;
        c->built = false;   // the next update builds afresh
    }
    return SPH_OK;
}

int sph_ctx_set_periodic(sph_ctx *c, int on, double xmin, double xmax) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_ctx_set_periodic");
    RESOLVE(c);
    if (on != 0 && on != 1) return set_error(SPH_ERR_ARG, "sph_ctx_set_periodic: on must be 0 or 1");
    if (on && !(xmax > xmin))
        return set_error(SPH_ERR_ARG, "sph_ctx_set_periodic: xmax must exceed xmin");
    if (on != c->periodic || (on && (xmin != c->pxmin || xmax != c->pxmax))) {
        c->periodic = on;
        c->pxmin = on ? xmin : 0.0;
        c->pxmax = on ? xmax : 0.0;
        c->built = false;   // the next update builds afresh
    }
    return SPH_OK;
}

int sph_ctx_set_bricks(sph_ctx *c, int on) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_ctx_set_bricks");
    RESOLVE(c);
    if (on != 0 && on != 1) return set_error(SPH_ERR_ARG, "sph_ctx_set_bricks: on must be 0 or 1");
    if (on != c->bricks_on) {
        c->bricks_on = on;
        c->built = false;   // the next update builds afresh
    }
    return SPH_OK;
}

int sph_pair_pass_stats(sph_ctx *c, int64_t *out) {
    CHECK_CTX(c);
    if (!out) return set_error(SPH_ERR_ARG, "sph_pair_pass_stats: null out");
    out[0] = c->n_brick_passes;
    return SPH_OK;
}

int sph_nnps_stats(sph_ctx *c, int64_t *out) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_nnps_stats");
    if (!out) return set_error(SPH_ERR_ARG, "sph_nnps_stats: null out");
    RESOLVE(c);
    out[0] = c->n_full;
    out[1] = c->n_light;
    return SPH_OK;
}

int sph_nnps_deferred_stats(sph_ctx *c, int64_t *out) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_nnps_deferred_stats");
    if (!out) return set_error(SPH_ERR_ARG, "sph_nnps_deferred_stats: null out");
    RESOLVE(c);
    out[0] = c->n_deferred;
    out[1] = c->n_deferred_stale;
    return SPH_OK;
}

int sph_nnps_count(sph_ctx *c, int dst, int src, double radius_scale, int64_t *counts) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_nnps_count");
    if (!counts) return set_error(SPH_ERR_ARG, "sph_nnps_count: null counts");
    RESOLVE(c);
    return nnps_count(c, dst, src, radius_scale, counts);
}

int sph_nnps_fill(sph_ctx *c, int dst, int src, double radius_scale, const int64_t *offsets,
                  int64_t *index) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_nnps_fill");
    if (!offsets || !index) return set_error(SPH_ERR_ARG, "sph_nnps_fill: null output");
    RESOLVE(c);
    return nnps_fill(c, dst, src, radius_scale, offsets, index);
}

int sph_nbr_lists(sph_ctx *c, int dst, const int *srcs, int nsrc) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_nbr_lists");
    RESOLVE(c);
    return build_lists(c, dst, srcs, nsrc);
}

int sph_refresh_state(sph_ctx *c, int array, const sph_array_view *view) {
    CHECK_CTX(c);
    if (!view) return set_error(SPH_ERR_ARG, "sph_refresh_state: null view");
    if (c->recording) return record_refresh(c, array, view);
    RESOLVE(c);
    return refresh_state(c, array, view);
}

int sph_density(sph_ctx *c, int dst, const int *srcs, int nsrc, const sph_density_params *prm,
                double *rho_out, double *p_out, double *cs_out) {
    CHECK_CTX(c);
    if (nsrc > 0 && !srcs) return set_error(SPH_ERR_ARG, "sph_density: null sources");
    if (prm && prm->tait && (!p_out || !cs_out))
        return set_error(SPH_ERR_ARG, "sph_density: Tait needs p and cs outputs");
    if (c->recording) return record_density(c, dst, srcs, nsrc, prm, rho_out, p_out, cs_out);
    return launch_density(c, dst, srcs, nsrc, prm, rho_out, p_out, cs_out);
}

int sph_rates(sph_ctx *c, int dst, const sph_source_term *terms, int nterms,
              const sph_rates_params *prm, double *const *acc_out, double *const *pos_out,
              int accumulate) {
    CHECK_CTX(c);
    if (nterms > 0 && !terms) return set_error(SPH_ERR_ARG, "sph_rates: null terms");
    if (c->recording) return record_rates(c, dst, terms, nterms, prm, acc_out, pos_out, accumulate);
    return launch_rates(c, dst, terms, nterms, prm, acc_out, pos_out, accumulate);
}

int sph_tait(sph_ctx *c, int64_t n, const double *rho, const int64_t *tag, double co, double ro,
             double gamma, double *p_out, double *cs_out) {
    CHECK_CTX(c);
    if (c->recording) return record_tait(c, n, rho, tag, co, ro, gamma, p_out, cs_out);
    return launch_tait(c, n, rho, tag, co, ro, gamma, p_out, cs_out);
}

int sph_adke_smoothing(sph_ctx *c, int64_t n, int64_t nreal, const int64_t *tag,
                       const double *rhop, double h0, double k, double eps, double *h_out) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_adke_smoothing");
    return launch_adke_smoothing(c, n, nreal, tag, rhop, h0, k, eps, h_out);
}

int sph_adke_conduction(sph_ctx *c, int64_t nreal, const int64_t *tag, const double *cs,
                        const double *h, const double *div, double g1, double g2,
                        double *q_out) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_adke_conduction");
    return launch_adke_conduction(c, nreal, tag, cs, h, div, g1, g2, q_out);
}

int sph_const_rates(sph_ctx *c, int kind, int64_t n, const int64_t *tag, const double *g3,
                    const double *u, const double *v, const double *w, int nout,
                    double *const *out) {
    CHECK_CTX(c);
    if (c->recording) return record_const(c, kind, n, tag, g3, u, v, w, nout, out);
    return launch_const_rates(c, kind, n, tag, g3, u, v, w, nout, out);
}

int sph_integrate(sph_ctx *c, int64_t n, const sph_axpy_line *lines, int nlines) {
    CHECK_CTX(c);
    if (c->recording) return record_integrate(c, n, lines, nlines);
    RESOLVE(c);
    return launch_integrate(c, n, lines, nlines);
}

int sph_invariants(sph_ctx *c, const sph_array_view *a, double *out) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_invariants");
    RESOLVE(c);
    return invariants(c, a, out);
}

int sph_batch_create(sph_batch **out) {
    if (!out) return set_error(SPH_ERR_ARG, "sph_batch_create: null out");
    sph_batch *b = new (std::nothrow) sph_batch();
    if (!b) return set_error(SPH_ERR_ARG, "sph_batch_create: out of host memory");
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete b;
        return cuda_check(e, "sph_batch_create: stream");
    }
    int rc = sph_ctx_create(3, &b->ctx);
    if (rc) {
        cudaStreamDestroy(b->stream);
        delete b;
        return rc;
    }
    b->ctx->stream = b->stream;
    *out = b;
    return SPH_OK;
}

int sph_batch_destroy(sph_batch *b) {
    if (!b) return SPH_OK;
    cudaStreamSynchronize(b->stream);
    batch_free(b);
    sph_ctx_destroy(b->ctx);
    cudaStreamDestroy(b->stream);
    delete b;
    return SPH_OK;
}

int sph_batch_setup(sph_batch *b, const sph_array_view *all, const sph_batch_instance *inst,
                    int ninst, const sph_batch_recipe *recipe) {
    if (!b) return set_error(SPH_ERR_ARG, "null sph_batch");
    if (b->ready) return set_error(SPH_ERR_STATE, "sph_batch_setup: batch already set up");
    return batch_setup(b, all, inst, ninst, recipe);
}

int sph_batch_step(sph_batch *b, int nsteps, int use_graph) {
    if (!b) return set_error(SPH_ERR_ARG, "null sph_batch");
    return batch_step(b, nsteps, use_graph);
}

int sph_batch_sync(sph_batch *b) {
    if (!b) return set_error(SPH_ERR_ARG, "null sph_batch");
    SPH_CUDA(cudaStreamSynchronize(b->stream));
    return SPH_OK;
}

int sph_batch_stream(sph_batch *b, void **out) {
    if (!b || !out) return set_error(SPH_ERR_ARG, "sph_batch_stream: null argument");
    *out = (void *)b->stream;
    return SPH_OK;
}

int sph_batch_pair_counts(sph_batch *b, uint64_t *out) {
    if (!b || !out) return set_error(SPH_ERR_ARG, "sph_batch_pair_counts: null argument");
    return batch_pair_counts(b, (unsigned long long *)out);
}

int sph_batch_stats(sph_batch *b, int64_t *out) {
    if (!b || !out) return set_error(SPH_ERR_ARG, "sph_batch_stats: null argument");
    out[0] = b->regrids;
    out[1] = b->total_cells;
    out[2] = (int64_t)b->h_steps;
    out[3] = (int64_t)b->groups.size();
    return SPH_OK;
}

int sph_batch_error_word(sph_batch *b, unsigned *out) {
    if (!b || !out) return set_error(SPH_ERR_ARG, "sph_batch_error_word: null argument");
    if (!b->d_err) { *out = 0; return SPH_OK; }
    unsigned h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, b->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_err, 0, sizeof(unsigned), b->stream);
    if (e != cudaSuccess) return cuda_check(e, "sph_batch_error_word");
    *out = h;
    return SPH_OK;
}

int sph_error_word(sph_ctx *c, unsigned *out) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_error_word");
    if (!out) return set_error(SPH_ERR_ARG, "sph_error_word: null out");
    RESOLVE(c);
    unsigned h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream);
    if (e != cudaSuccess) return cuda_check(e, "sph_error_word");
    *out = h;
    return SPH_OK;
}

int sph_mean_neighbours(sph_ctx *c, int dst, int src, double *out) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_mean_neighbours");
    if (!out) return set_error(SPH_ERR_ARG, "sph_mean_neighbours: null out");
    RESOLVE(c);
    if (!c->built || dst < 0 || dst >= (int)c->arrays.size())
        return set_error(SPH_ERR_STATE, "sph_mean_neighbours: no neighbour build");
    int64_t n = c->arrays[dst].n;
    if (n == 0) { *out = 0.0; return SPH_OK; }
    if (n + 1 > c->cnt_cap) {
        cudaFree(c->d_cnt);
        c->d_cnt = nullptr;
        SPH_CUDA(cudaMalloc(&c->d_cnt, sizeof(int64_t) * (n + 1)));
        c->cnt_cap = n + 1;
    }
    int rc = nnps_count(c, dst, src, c->grid.radius_scale, c->d_cnt);
    if (rc) return rc;
    unsigned long long *acc = (unsigned long long *)(c->d_part);
    SPH_CUDA(cudaMemsetAsync(acc, 0, sizeof(unsigned long long), c->stream));
    k_sum_i64<<<grid_blocks(n, 256, 2), 256, 0, c->stream>>>(c->d_cnt, n, acc);
    count_launch();
    SPH_LAUNCH_CHECK("k_sum_i64");
    unsigned long long h = 0;
    SPH_CUDA(cudaMemcpyAsync(&h, acc, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    SPH_CUDA(cudaStreamSynchronize(c->stream));
    *out = (double)h / (double)n;
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// learned momentum closure
// ---------------------------------------------------------------------------
static bool mlp_model_ok(const sph_mlp_model *m) {
    return m && m->params && m->w1 && m->w2 && m->w2t && m->w3;
}

int sph_mlp_features(sph_ctx *c, int dst, int src, const sph_mlp_feature_params *prm,
                     uint16_t *out_bf16, float *out_f32) {
    CHECK_CTX(c);
    NOT_RECORDING(c, "sph_mlp_features");
    return launch_features(c, dst, src, prm, out_bf16, out_f32);
}

int sph_mlp_sync(const sph_mlp_model *m, void *stream) {
    if (!mlp_model_ok(m)) return set_error(SPH_ERR_ARG, "sph_mlp_sync: incomplete model");
    return mlp_sync(m, (cudaStream_t)stream);
}

int sph_mlp_forward(const sph_mlp_model *m, const uint16_t *x, int64_t n, float *y, float *z1,
                    float *z2, uint16_t *h1, uint16_t *h2, uint32_t *err, void *stream) {
    if (!mlp_model_ok(m) || !x || !y || !err || n < 0)
        return set_error(SPH_ERR_ARG, "sph_mlp_forward: null argument");
    return mlp_forward(m, x, n, y, z1, z2, h1, h2, err, (cudaStream_t)stream);
}

int sph_mlp_backward_scratch(int64_t n, int64_t *floats) {
    if (!floats || n < 0) return set_error(SPH_ERR_ARG, "sph_mlp_backward_scratch: bad argument");
    *floats = mlp_backward_scratch(n);
    return SPH_OK;
}

int sph_mlp_backward(const sph_mlp_model *m, const uint16_t *x, const uint16_t *h1,
                     const uint16_t *h2, const float *z1, const float *z2, const float *y,
                     const float *target, int64_t n, float inv_count, float *grad, float *loss,
                     float *scratch, uint32_t *err, void *stream) {
    if (!mlp_model_ok(m) || !x || !h1 || !h2 || !z1 || !z2 || !y || !target || !grad ||
        !scratch || !err)
        return set_error(SPH_ERR_ARG, "sph_mlp_backward: null argument");
    return mlp_backward(m, x, h1, h2, z1, z2, y, target, n, inv_count, grad, loss, scratch, err,
                        (cudaStream_t)stream);
}

int sph_mlp_adam(const sph_mlp_model *m, const float *grad, float *mom, float *vel, float lr,
                 float beta1, float beta2, float eps, int step, void *stream) {
    if (!mlp_model_ok(m) || !grad || !mom || !vel)
        return set_error(SPH_ERR_ARG, "sph_mlp_adam: null argument");
    return mlp_adam(m, grad, mom, vel, lr, beta1, beta2, eps, step, (cudaStream_t)stream);
}

int sph_mlp_apply(sph_ctx *c, int dst, const float *y, double c0, const double *scale,
                  const double *mean, double *const *acc, int accumulate) {
    CHECK_CTX(c);
    if (dst < 0 || dst >= (int)c->arrays.size() || !y || !scale || !mean || !acc)
        return set_error(SPH_ERR_ARG, "sph_mlp_apply: bad argument");
    const sph_array_view &v = c->arrays[dst].view;
    if (!v.h) return set_error(SPH_ERR_ARG, "sph_mlp_apply: destination has no h");
    return mlp_apply(v.n, y, v.tag, v.h, c0, scale, mean, acc, accumulate, c->stream);
}

int sph_mlp_targets(int64_t n, const double *ax, const double *ay, const double *h, double c0,
                    const double *mean, const double *inv_std, float *out, void *stream) {
    if (!ax || !ay || !h || !mean || !inv_std || !out || c0 <= 0.0)
        return set_error(SPH_ERR_ARG, "sph_mlp_targets: bad argument");
    return mlp_targets(n, ax, ay, h, c0, mean, inv_std, out, (cudaStream_t)stream);
}

int sph_selftest_conversions(int64_t n, int64_t *mismatches) {
    return selftest_conversions(n, mismatches);
}

}  // extern "C"

