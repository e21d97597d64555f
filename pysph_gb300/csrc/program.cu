// Step programs (sm_103a): one integrator step recorded once and replayed as
// a CUDA graph.
//
// The reference advances a simulation with Python calls per calc and per
// NumPy line (solver/integrator.py:432-645, solver/solver.py:457-508).  Here
// the calls of one step (neighbour updates, density and rates passes, Tait,
// constant rates, integrator lines) are recorded as a program; while the
// neighbour build stays the same (light refreshes only), the program is
// captured once into a CUDA graph in which every launch after a light
// refresh is gated on the refresh's stale word, and the whole step becomes
// one graph launch.  After the launch the host reads the step's status
// block (published into mapped memory by the graph's last node): a jump is
// reported as by the calls themselves; a light refresh that found the lists
// stale (its bit in status[3]) made every later launch return at once, so
// the step resumes there -- a full neighbour build, then the rest of the
// step's calls eagerly -- with results identical to the eager step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "sph_internal.cuh"

namespace sphgb {

enum OpKind { kOpUpdate, kOpBuild, kOpDensity, kOpRates, kOpTait, kOpConst, kOpIntegrate, kOpRefresh };

struct StepOp {
    OpKind kind;
    // update / build
    std::vector<sph_array_view> views;
    double cell_size = 0, radius_scale = 0;
    int subdiv = 1, check_jump = 0;
    // density / rates
    int dst = 0;
    std::vector<int> srcs;
    sph_density_params dprm{};
    double *rho = nullptr, *p = nullptr, *cs = nullptr;
    std::vector<sph_source_term> terms;
    sph_rates_params rprm{};
    double *acc[3] = {nullptr, nullptr, nullptr}, *pos[3] = {nullptr, nullptr, nullptr};
    int accumulate = 0;
    // tait / const rates / integrate / refresh
    int64_t n = 0;
    const double *rho_in = nullptr;
    const int64_t *tag = nullptr;
    double co = 0, ro = 0, gamma = 0;
    int ckind = 0, nout = 0;
    double g3[3] = {0, 0, 0};
    const double *u = nullptr, *v = nullptr, *w = nullptr;
    double *out[3] = {nullptr, nullptr, nullptr};
    std::vector<sph_axpy_line> lines;
    int array = 0;
    sph_array_view view{};
};

}  // namespace sphgb

struct sph_step {
    sph_ctx *ctx = nullptr;
    std::vector<sphgb::StepOp> ops;
    cudaGraphExec_t exec = nullptr;
    long long graph_build = -1;    // neighbour build the graph belongs to
    long long attempt_build = -1;  // build of the last capture attempt
    // the last step ran without a full build: the flow is in the regime of
    // light refreshes that a graph serves (a flow that rebuilds at every
    // update is left to the eager calls)
    bool settled = false;
    int updates = 0;               // light refreshes in one step
    int launches = 0;              // kernels of one replay
    long long passes = 0;          // brick-staged pair passes of one replay
    // host state of the context after a captured step (restored after a replay)
    std::vector<bool> st_fresh;
    std::vector<double> st_tait_f;
    cudaEvent_t done = nullptr;
    // device time of the replays (CUDA events around each graph launch)
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    double replay_us = 0.0;
    // the stream of the steps when the context's is the legacy default
    // stream (which cannot be captured); a blocking stream, so it is ordered
    // with the default stream's work
    cudaStream_t stream = nullptr;
    long long n_graph = 0, n_eager = 0, n_resumed = 0, n_captures = 0;
    long long n_attempts = 0;      // capture attempts
    long long n_updates = 0;       // captures that updated the executable in place
    int last_fail = 0;             // why the last attempt found no graph (see sph_step_stats)
    // capture back-off: a flow whose lists go stale within a step or two of
    // every full build spends a capture per build for no replay; after a
    // graph that never ran a whole step the next 1, 2, 4 .. 64 capture
    // opportunities are skipped (reset by a graph that ran two steps)
    int lifetime = 0;              // whole-step replays of the current graph
    bool judged = true;            // the last graph's lifetime was taken into account
    int backoff = 0, skip = 0;
    double skin = -1.0;            // the list skin the back-off was learnt with
};

namespace sphgb {

namespace {

int run_op(sph_ctx *ctx, const StepOp &o) {
    switch (o.kind) {
        case kOpUpdate: {
            int rebuilt = 0;
            {
                const int rc = resolve_pending(ctx);
                if (rc) return rc;
            }
            return nnps_update(ctx, o.views.data(), (int)o.views.size(), o.cell_size,
                               o.radius_scale, o.subdiv, o.check_jump, &rebuilt);
        }
        case kOpBuild: {
            const int rc = resolve_pending(ctx);
            if (rc) return rc;
            return nnps_build(ctx, o.views.data(), (int)o.views.size(), o.cell_size,
                              o.radius_scale, o.subdiv, o.check_jump);
        }
        case kOpDensity:
            return launch_density(ctx, o.dst, o.srcs.data(), (int)o.srcs.size(), &o.dprm, o.rho,
                                  o.p, o.cs);
        case kOpRates:
            return launch_rates(ctx, o.dst, o.terms.data(), (int)o.terms.size(), &o.rprm, o.acc,
                                o.pos, o.accumulate);
        case kOpTait:
            return launch_tait(ctx, o.n, o.rho_in, o.tag, o.co, o.ro, o.gamma, o.p, o.cs);
        case kOpConst:
            return launch_const_rates(ctx, o.ckind, o.n, o.tag, o.g3, o.u, o.v, o.w, o.nout, o.out);
        case kOpIntegrate: {
            const int rc = resolve_pending(ctx);
            if (rc) return rc;
            return launch_integrate(ctx, o.n, o.lines.data(), (int)o.lines.size());
        }
        case kOpRefresh: {
            const int rc = resolve_pending(ctx);
            if (rc) return rc;
            return refresh_state(ctx, o.array, &o.view);
        }
    }
    return set_error(SPH_ERR_ARG, "step program: unknown call");
}

int run_eager(sph_step *s, size_t from) {
    for (size_t i = from; i < s->ops.size(); ++i) {
        const int rc = run_op(s->ctx, s->ops[i]);
        if (rc) return rc;
    }
    return SPH_OK;
}

// The graph no longer matches the build; its executable is kept, so that
// the next capture can update it in place (cudaGraphExecUpdate, far cheaper
// than instantiating) when its topology has not changed.
void drop_graph(sph_step *s) { s->graph_build = -1; }

void destroy_graph(sph_step *s) {
    if (s->exec) cudaGraphExecDestroy(s->exec);
    s->exec = nullptr;
    s->graph_build = -1;
}

// Capture the program into a graph for the current neighbour build.  The
// launchers, with ctx->capturing set, take every light-refresh path without
// synchronising and flag anything that would need the host (a full build, a
// list build, a pending status) as capture_failed.
int capture(sph_step *s) {
    sph_ctx *ctx = s->ctx;
    drop_graph(s);
    if (!ctx->built || ctx->pending || ctx->stream == 0) return SPH_OK;
    const long long build = ctx->build_id;
    const long long launches0 = [] { int64_t v; sph_launch_count(&v); return (long long)v; }();
    const long long passes0 = ctx->n_brick_passes;
    const long long light0 = ctx->n_light;
    // host state the capture may change without running anything
    std::vector<bool> fresh0;
    std::vector<double> tait0;
    std::vector<sph_array_view> views0;
    for (const auto &A : ctx->arrays) {
        fresh0.push_back(A.st_fresh);
        tait0.push_back(A.st_tait_f);
        views0.push_back(A.view);
    }
    cudaGraph_t graph = nullptr;
    SPH_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
    ctx->capturing = true;
    ctx->capture_failed = false;
    ctx->capture_fail_site = 0;
    s->n_attempts += 1;
    ctx->gate = ctx->d_status + kStaleWord;
    int rc = SPH_OK;
    // error word, displacement, stale word, stale bits
    cudaError_t e = cudaMemsetAsync(ctx->d_status, 0, 4 * sizeof(unsigned), ctx->stream);
    if (e != cudaSuccess) rc = cuda_check(e, "cudaMemsetAsync (step status)");
    int u = 0;
    for (size_t i = 0; !rc && !ctx->capture_failed && i < s->ops.size(); ++i) {
        const StepOp &o = s->ops[i];
        if (o.kind == kOpUpdate) {
            if (u >= 32) {
                ctx->capture_failed = true;
                ctx->capture_fail_site = 6;
                break;
            }
            ctx->capture_stale_bit = 1u << u;
            ++u;
        }
        if (o.kind == kOpBuild) {
            ctx->capture_failed = true;
            ctx->capture_fail_site = 7;
            break;
        }
        rc = run_op(ctx, o);
        ctx->capture_stale_bit = 0;
    }
    if (!rc && !ctx->capture_failed)
        rc = publish_words(ctx, ctx->d_status, ctx->hd_status, kListWord0);
    ctx->capturing = false;
    ctx->gate = nullptr;
    e = cudaStreamEndCapture(ctx->stream, &graph);
    const int rc_capture = rc;
    bool ok = !rc && !ctx->capture_failed && e == cudaSuccess && graph != nullptr &&
              ctx->build_id == build;
    if (ok) {
        bool made = false;
        if (s->exec) {
            // same calls, other arguments: update the executable in place
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(s->exec, graph, &info) == cudaSuccess) {
                made = true;
                s->n_updates += 1;
            } else {
                cudaGetLastError();
                cudaGraphExecDestroy(s->exec);
                s->exec = nullptr;
            }
        }
        if (!made) {
            e = cudaGraphInstantiate(&s->exec, graph, 0);
            made = e == cudaSuccess;
            if (!made) s->exec = nullptr;
        }
        ok = made;
    }
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    // an error inside the capture (a call that cannot be captured) leaves
    // this build without a graph: the steps run their calls eagerly
    rc = SPH_OK;
    // the capture ran nothing: undo its host-side counters
    {
        int64_t v;
        sph_launch_count(&v);
        s->launches = (int)(v - launches0);
        count_launch(-s->launches);
    }
    s->passes = ctx->n_brick_passes - passes0;
    ctx->n_brick_passes = passes0;
    s->updates = u;
    ctx->n_light = light0;
    if (!ok || !s->exec) {
        s->last_fail = ctx->capture_failed ? ctx->capture_fail_site
                       : (rc_capture ? 8 : (ctx->build_id != build ? 9 : 10));
        drop_graph(s);
        for (size_t a = 0; a < ctx->arrays.size() && a < fresh0.size(); ++a) {
            ctx->arrays[a].st_fresh = fresh0[a];
            ctx->arrays[a].st_tait_f = tait0[a];
            ctx->arrays[a].view = views0[a];
        }
        return SPH_OK;
    }
    s->graph_build = build;
    s->st_fresh.clear();
    s->st_tait_f.clear();
    for (const auto &A : ctx->arrays) {
        s->st_fresh.push_back(A.st_fresh);
        s->st_tait_f.push_back(A.st_tait_f);
    }
    s->n_captures += 1;
    return SPH_OK;
}

// One step as a graph launch; resumes eagerly after a stale light refresh.
int replay(sph_step *s) {
    sph_ctx *ctx = s->ctx;
    SPH_CUDA(cudaEventRecord(s->t0, ctx->stream));
    SPH_CUDA(cudaGraphLaunch(s->exec, ctx->stream));
    SPH_CUDA(cudaEventRecord(s->t1, ctx->stream));
    SPH_CUDA(cudaEventSynchronize(s->t1));
    {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, s->t0, s->t1) == cudaSuccess) s->replay_us += 1e3 * ms;
    }
    count_launch(s->launches);
    ctx->n_brick_passes += s->passes;
    for (size_t a = 0; a < ctx->arrays.size() && a < s->st_fresh.size(); ++a) {
        ctx->arrays[a].st_fresh = s->st_fresh[a];
        ctx->arrays[a].st_tait_f = s->st_tait_f[a];
    }
    list_maxima_collect(ctx);
    const unsigned err = ctx->h_status[0];
    const unsigned bits = ctx->h_status[kStaleBitsWord];
    if (err & SPH_EFLAG_JUMP) {
        ctx->built = false;
        drop_graph(s);
        return set_error(SPH_ERR_JUMP, "Particle moved by more than one cell width");
    }
    if (!bits) {
        ctx->n_light += s->updates;
        s->n_graph += 1;
        s->lifetime += 1;
        return SPH_OK;
    }
    // the first stale light refresh: a full build in its place, then the
    // rest of the step as eager calls
    const int u = __builtin_ctz(bits);
    ctx->n_light += u;
    int seen = 0;
    size_t at = 0;
    for (; at < s->ops.size(); ++at)
        if (s->ops[at].kind == kOpUpdate && seen++ == u) break;
    const StepOp &o = s->ops[at];
    ctx->n_deferred_stale += 1;
    int rc = nnps_build(ctx, o.views.data(), (int)o.views.size(), o.cell_size, o.radius_scale,
                        o.subdiv, 0);
    if (!rc) rc = run_eager(s, at + 1);
    s->n_resumed += 1;
    drop_graph(s);
    return rc;
}

StepOp &append(sph_ctx *ctx, OpKind k) {
    ctx->recording->ops.emplace_back();
    StepOp &o = ctx->recording->ops.back();
    o.kind = k;
    return o;
}

}  // namespace

// ---------------------------------------------------------------------------
// recording (called by the C ABI entry points while a program is recorded)
// ---------------------------------------------------------------------------
int record_update(sph_ctx *ctx, bool build, const sph_array_view *arrays, int narrays,
                  double cell_size, double radius_scale, int subdiv, int check_jump) {
    if (narrays <= 0 || !arrays) return set_error(SPH_ERR_ARG, "step program: update without arrays");
    StepOp &o = append(ctx, build ? kOpBuild : kOpUpdate);
    o.views.assign(arrays, arrays + narrays);
    o.cell_size = cell_size;
    o.radius_scale = radius_scale;
    o.subdiv = subdiv;
    o.check_jump = check_jump;
    return SPH_OK;
}

int record_density(sph_ctx *ctx, int dst, const int *srcs, int nsrc, const sph_density_params *prm,
                   double *rho, double *p, double *cs) {
    if (!prm || nsrc < 0 || (nsrc > 0 && !srcs))
        return set_error(SPH_ERR_ARG, "step program: bad density call");
    StepOp &o = append(ctx, kOpDensity);
    o.dst = dst;
    o.srcs.assign(srcs, srcs + nsrc);
    o.dprm = *prm;
    o.rho = rho; o.p = p; o.cs = cs;
    return SPH_OK;
}

int record_rates(sph_ctx *ctx, int dst, const sph_source_term *terms, int nterms,
                 const sph_rates_params *prm, double *const *acc, double *const *pos,
                 int accumulate) {
    if (!prm || nterms < 0 || (nterms > 0 && !terms))
        return set_error(SPH_ERR_ARG, "step program: bad rates call");
    StepOp &o = append(ctx, kOpRates);
    o.dst = dst;
    o.terms.assign(terms, terms + nterms);
    o.rprm = *prm;
    for (int c = 0; c < 3; ++c) {
        o.acc[c] = acc ? acc[c] : nullptr;
        o.pos[c] = pos ? pos[c] : nullptr;
    }
    o.accumulate = accumulate;
    return SPH_OK;
}

int record_tait(sph_ctx *ctx, int64_t n, const double *rho, const int64_t *tag, double co,
                double ro, double gamma, double *p, double *cs) {
    StepOp &o = append(ctx, kOpTait);
    o.n = n; o.rho_in = rho; o.tag = tag; o.co = co; o.ro = ro; o.gamma = gamma;
    o.p = p; o.cs = cs;
    return SPH_OK;
}

int record_const(sph_ctx *ctx, int kind, int64_t n, const int64_t *tag, const double *g3,
                 const double *u, const double *v, const double *w, int nout, double *const *out) {
    if (nout < 0 || nout > 3 || (nout > 0 && !out))
        return set_error(SPH_ERR_ARG, "step program: bad constant-rates call");
    StepOp &o = append(ctx, kOpConst);
    o.ckind = kind; o.n = n; o.tag = tag;
    for (int c = 0; c < 3; ++c) o.g3[c] = g3 ? g3[c] : 0.0;
    o.u = u; o.v = v; o.w = w;
    o.nout = nout;
    for (int c = 0; c < nout; ++c) o.out[c] = out[c];
    return SPH_OK;
}

int record_integrate(sph_ctx *ctx, int64_t n, const sph_axpy_line *lines, int nlines) {
    if (nlines < 0 || (nlines > 0 && !lines))
        return set_error(SPH_ERR_ARG, "step program: bad integrate call");
    StepOp &o = append(ctx, kOpIntegrate);
    o.n = n;
    o.lines.assign(lines, lines + nlines);
    return SPH_OK;
}

int record_refresh(sph_ctx *ctx, int array, const sph_array_view *view) {
    StepOp &o = append(ctx, kOpRefresh);
    o.array = array;
    o.view = *view;
    return SPH_OK;
}

}  // namespace sphgb

namespace sphgb {
int run_steps(sph_step *s, int nsteps);
}

using namespace sphgb;

extern "C" {

int sph_step_begin(sph_ctx *ctx) {
    if (!ctx) return set_error(SPH_ERR_ARG, "sph_step_begin: null context");
    if (ctx->recording) return set_error(SPH_ERR_STATE, "sph_step_begin: already recording");
    sph_step *s = new (std::nothrow) sph_step();
    if (!s) return set_error(SPH_ERR_ARG, "sph_step_begin: out of host memory");
    cudaError_t e = cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&s->t0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->t1);
    if (e != cudaSuccess) {
        if (s->done) cudaEventDestroy(s->done);
        if (s->t0) cudaEventDestroy(s->t0);
        delete s;
        return cuda_check(e, "sph_step_begin");
    }
    s->ctx = ctx;
    ctx->recording = s;
    return SPH_OK;
}

int sph_step_end(sph_ctx *ctx, sph_step **out) {
    if (!ctx || !out) return set_error(SPH_ERR_ARG, "sph_step_end: null argument");
    if (!ctx->recording) return set_error(SPH_ERR_STATE, "sph_step_end: not recording");
    *out = ctx->recording;
    ctx->recording = nullptr;
    return SPH_OK;
}

int sph_step_run(sph_step *s, int nsteps) {
    if (!s || nsteps < 0) return set_error(SPH_ERR_ARG, "sph_step_run: bad arguments");
    sph_ctx *ctx = s->ctx;
    if (ctx->recording) return set_error(SPH_ERR_STATE, "sph_step_run: the context is recording");
    cudaStream_t caller = ctx->stream;
    if (caller == 0) {
        if (!s->stream) SPH_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamDefault));
        const int rc = resolve_pending(ctx);   // a pending refresh belongs to the old stream
        if (rc) return rc;
        ctx->stream = s->stream;
    }
    const int rc = run_steps(s, nsteps);
    ctx->stream = caller;
    return rc;
}

}  // extern "C"

namespace sphgb {

int run_steps(sph_step *s, int nsteps) {
    sph_ctx *ctx = s->ctx;
    for (int k = 0; k < nsteps; ++k) {
        int rc;
        // another list skin is another regime: forget the back-off
        if (ctx->skin_frac != s->skin) {
            s->skin = ctx->skin_frac;
            s->backoff = s->skip = 0;
            s->judged = true;
        }
        // a graph (or its capture) starts from a resolved neighbour update;
        // eager steps leave a pending refresh to their first pass
        if (ctx->pending && (s->settled || (s->exec && s->graph_build == ctx->build_id))) {
            rc = resolve_pending(ctx);
            if (rc) return rc;
        }
        // one capture attempt per build, after a step that needed no full
        // build (the first eager pass of a build writes its lists)
        if (ctx->built && !ctx->pending && s->settled && s->graph_build != ctx->build_id &&
            s->attempt_build != ctx->build_id && !s->ops.empty()) {
            s->attempt_build = ctx->build_id;
            if (!s->judged) {
                s->judged = true;
                if (s->lifetime == 0) s->backoff = std::min(64, std::max(1, 2 * s->backoff));
                else if (s->lifetime >= 2) s->backoff = 0;
                s->skip = s->backoff;
            }
            if (s->skip > 0) {
                --s->skip;
            } else {
                rc = capture(s);
                if (rc) return rc;
                if (s->graph_build == ctx->build_id) {
                    s->judged = false;
                    s->lifetime = 0;
                } else if (s->last_fail >= 2 && s->last_fail <= 5) {
                    // a neighbour list of this build was not built yet (the
                    // refresh resolved at the step's start rebuilt): the
                    // eager step builds it, the next step tries again
                    s->attempt_build = -1;
                }
            }
        }
        const long long full0 = ctx->n_full;
        if (s->exec && s->graph_build == ctx->build_id && ctx->built && !ctx->pending) {
            rc = replay(s);
        } else {
            rc = run_eager(s, 0);
            s->n_eager += 1;
        }
        if (rc) return rc;
        // settled: no full build inside the step (a refresh still pending is
        // judged when the next step resolves it)
        s->settled = ctx->n_full == full0;
    }
    return SPH_OK;
}

}  // namespace sphgb

extern "C" {

int sph_step_stats(sph_step *s, int64_t *out) {
    if (!s || !out) return set_error(SPH_ERR_ARG, "sph_step_stats: null argument");
    out[0] = s->n_graph;
    out[1] = s->n_eager;
    out[2] = s->n_resumed;
    out[3] = s->n_captures;
    out[4] = (int64_t)s->ops.size();
    out[5] = s->launches;
    out[6] = (int64_t)(s->replay_us + 0.5);
    out[7] = s->n_attempts;
    out[8] = s->last_fail;
    out[9] = s->n_updates;
    return SPH_OK;
}

int sph_step_destroy(sph_step *s) {
    if (!s) return SPH_OK;
    if (s->ctx && s->ctx->recording == s) s->ctx->recording = nullptr;
    destroy_graph(s);
    if (s->done) cudaEventDestroy(s->done);
    if (s->t0) cudaEventDestroy(s->t0);
    if (s->t1) cudaEventDestroy(s->t1);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SPH_OK;
}

}  // extern "C"
