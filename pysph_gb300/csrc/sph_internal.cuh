// Internal declarations of the pysph_gb300 CUDA library (sm_103a).
//
// Data layout (per particle array, per neighbour build):
//   original order (caller-owned FP64 SoA):  x y z u v w m h rho p cs [nx..tz] tag
//   sorted order (context-owned, cell-major, deterministic within a cell):
//     perm[s]  -> original index of sorted slot s          int32
//     skey[s]  -> dense-grid cell of slot s                int32
//     pm[s]    =  (xi_x, xi_y, xi_z, m)   cell-local FP32 offsets and mass: the
//                 one 16-byte record per neighbour of the pair passes
//     scx[s]   =  cx                       dense x cell (FP32, exact), fixed
//                 between full builds
//     velh[s]  =  (u, v, w, h)                              FP32
//     st[s]    =  (rho, p/rho^2, cs, m)                     FP32
//     nrm[s], tan[s] (walls only)
//   per array dense cell table cstart[ncells+1] (exclusive prefix of counts).
// A row of 2K+1 cells along x is contiguous in the sorted arrays, so one
// (dy, dz) stencil row is a single index range [cstart[c-K], cstart[c+K+1]).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "pysph_gb300.h"

namespace sphgb {

constexpr int kPairBlock = 128; // threads per block of the pair kernels
// (dst, src) lists whose maxima are tracked: the list-streaming lists of
// slots [0, na^2) and the brick-staged lists of slots [na^2, 2 na^2)
constexpr int kMaxListSlots = 128;
// device status block read back with one copy: [0] error word, [1] largest
// squared displacement (float bits), [2] stale-list flags of the last light
// refresh, [3] stale bits of a replayed step, [kListWord0 + i] largest count
// of list slot i
constexpr int kListWord0 = 4;
constexpr int kStatusWords = kListWord0 + kMaxListSlots;
// [2]: the lists cannot serve the last light refresh (a particle moved by
// half the skin, an h changed, a jump, or a list outgrew its capacity);
// a gated pair pass returns at once
constexpr unsigned kStaleLists = 1u;
constexpr int kStaleWord = 2;
// [3]: in a replayed step, bit u set when the u-th light refresh of the
// step found the lists stale (the step resumes after the first such one)
constexpr int kStaleBitsWord = 3;

struct Grid {
    int bx0 = 0, by0 = 0, bz0 = 0; // origin of the dense grid (internal cell coords)
    int nx = 1, ny = 1, nz = 1;    // dense grid dims
    int kx = 1, ky = 0, kz = 0;    // stencil half widths (cells)
    int64_t ncells = 1;
    double cs = 1.0;               // internal cell size
    double inv_cs = 1.0;
    float cs_f = 1.f;
    double radius_scale = 2.0;
    int uniform_h = 0;             // every particle of every array has the same h
    float h_uniform = 1.f;
    int64_t cell_base = 0;         // first cell of this grid in a shared cell table
    // neighbour-list skin (absolute): lists hold every source within
    // radius_scale h + skin of the destination at the build, the passes that
    // stream a list keep the exact neighbours; 0 = lists are exact
    float skin = 0.f;
    // variable h (VarHNbrParticleLocator): j is also a neighbour of i when
    // i lies within the radius of j; reach2 is the squared largest list
    // radius (radius_scale max h + skin, with a margin), the pruning radius
    int symmetric = 0;
    float reach2 = 0.f;
    // periodic x axis (the reference's PeriodicDomain, cell.pyx:1277-1376):
    // particles are binned at their image in [pxmin, pxmin + plen), measured
    // from pxmin; the grid spans exactly the period (bx0 = 0, nx cells of
    // size plen / nx) and a stencil row that leaves it continues at the other
    // end, where the sources are the images shifted by -+plen
    int periodic = 0;
    double pxmin = 0.0, plen = 0.0;
};

// FP64 -> FP32, round to nearest even, by integer operations only: on GB300
// the FP64 pipe, which also executes the FP64 conversions, runs at a small
// fraction of the FP32 rate (and a conversion left in the code under a
// predicate still takes its issue slot there).  The result equals
// __double2float_rn(x) for every non-NaN x, results below the normal FP32
// range (rounded to a subnormal or zero) and overflow to infinity included;
// a NaN gives a quiet NaN.
__device__ __forceinline__ float d2f_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u;
    const int E = (int)((hi >> 20) & 0x7ffu);
    const int e = E - 896;                             // FP32 biased exponent
    const unsigned m23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    const unsigned up = (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) ? 1u : 0u;
    // a carry out of the mantissa raises the exponent (to infinity from 254)
    unsigned r = sign | (((unsigned)e << 23) + m23 + up);
    if (e >= 255) {
        const bool nan = E == 0x7ff && ((hi & 0xfffffu) | lo) != 0u;
        r = nan ? 0x7fffffffu : (sign | 0x7f800000u);
    } else if (e <= 0) {
        // |x| < 2^-126: the FP32 subnormal m 2^-149 nearest to x, with the
        // full 53-bit significand shifted right by 30 - e (beyond 54 places
        // it is below half the smallest subnormal: zero; a double zero or
        // subnormal lands there too)
        const int sh = 30 - e;
        const unsigned long long M = (b & 0xfffffffffffffull) | (1ull << 52);
        unsigned q = 0u;
        if (sh <= 54) {
            const unsigned long long lowm = M & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
            q = (unsigned)(M >> sh);
            q += (lowm > half || (lowm == half && (q & 1u))) ? 1u : 0u;
        }
        r = sign | q;
    }
    return __uint_as_float(r);
}

// int -> FP64 (exact) by integer operations, as d2f_rn
__device__ __forceinline__ double i2d_exact(int n) {
    if (n == 0) return 0.0;
    const unsigned long long sign = n < 0 ? (1ull << 63) : 0ull;
    const unsigned a = n < 0 ? 0u - (unsigned)n : (unsigned)n;
    const int e = 31 - __clz(a);                      // a in [2^e, 2^(e+1))
    const unsigned long long m = ((unsigned long long)a << (52 - e)) & ((1ull << 52) - 1ull);
    return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 1023) << 52) | m));
}

// floor(x * inv) with the product rounded in FP64: a real call, so that its
// FP64 instructions are issued only by the warps that take it
static __device__ __noinline__ int floor_cell_fp64(double x, double inv) {
    return (int)floor(x * inv);
}

// floor(x * inv) with the product rounded in FP64 (the reference's cell
// index), screened in FP32: the FP32 product is within |t| 2^-22 of it, so
// its floor is the same unless a cell boundary lies that close; only then
// the FP64 product.
__device__ __forceinline__ int floor_cell_screened(double x, double inv, float invf) {
    const float tf = d2f_rn(x) * invf;
    const float at = fabsf(tf);
    int c = __float2int_rd(tf);
    const float fr = tf - (float)c;
    const float tol = fmaf(at, 4.8e-7f, 1e-30f);
    if (!(at < 4194304.f && fr > tol && fr < 1.f - tol)) c = floor_cell_fp64(x, inv);
    return c;
}

// Binning coordinate along x: the position, or on a periodic axis the offset
// of its image in [pxmin, pxmin + plen) from pxmin.
__device__ __forceinline__ double bin_x(const Grid &g, double x) {
    if (!g.periodic) return x;
    double t = x - g.pxmin;
    t -= g.plen * floor(t / g.plen);
    return t;
}

// Grid x cell of binning coordinate xb (clamped into the period, where
// rounding can put xb on its upper end).
__device__ __forceinline__ int bin_cell_x(const Grid &g, double xb) {
    int c = (int)floor(xb * g.inv_cs) - g.bx0;
    if (g.periodic) c = min(max(c, 0), g.nx - 1);
    return c;
}

// The image of source coordinate xj that destination coordinate xi sees,
// given the FP32 separation rx = x_i - x_j(image): xj itself, or on a periodic
// axis xj +- plen (added in FP64 like the reference's ghost copies).
__device__ __forceinline__ double image_x(const Grid &g, double xj, double xi, float rx) {
    if (!g.periodic) return xj;
    const double s = rint((xi - xj - (double)rx) / g.plen);
    return s == 0.0 ? xj : __dadd_rn(xj, s * g.plen);
}

// Bricks of grid cells, the unit of work of the brick-staged pair passes:
// bx * by * bz cells per brick, nbx * nby * nbz bricks over the grid.
struct BrickGeom {
    int bx = 1, by = 1, bz = 1;
    int nbx = 1, nby = 1, nbz = 1;
    int64_t nbricks = 0;
};

struct ArraySnap {
    int64_t n = 0;
    int64_t cap = 0;
    sph_array_view view{};
    bool has_nrm = false;
    // st holds the arrays' current rho, p, cs (a light refresh leaves it
    // to the next density pass, or to a state refresh before a pass that
    // reads it)
    bool st_fresh = true;
    // st's cs was written by the Tait equation with gamma = 7 from st's rho:
    // cs = st_tait_f rho^3 (co / ro^3); 0 when st came from anything else
    double st_tait_f = 0.0;
    int *key = nullptr;   // original order, dense cell index
    int *perm = nullptr;  // sorted -> original
    int *skey = nullptr;  // sorted: cell
    float4 *velh = nullptr, *st = nullptr, *nrm = nullptr, *tan = nullptr;
    float4 *pm = nullptr;
    float *scx = nullptr;   // sorted: dense x cell
    int *cstart = nullptr; // ncells + 1
    int *cursor = nullptr; // ncells
    int64_t cell_cap = 0;
    int *refcell = nullptr; // original order, 3 ints per particle (jump check)
    int64_t ref_n = -1;     // particle count the refcell entries belong to
    float4 *pm0 = nullptr; // pm at the last full build, in original order (skin lists)
    int *inv = nullptr;      // original -> sorted slot of the last full build
    int64_t pm0_cap = 0;
    // brick tables of the last full build: exclusive prefix of the
    // destinations per brick (nbricks + 1), the largest count of source
    // particles a brick stages and of destinations in one brick
    int *bdst = nullptr;
    int64_t bdst_cap = 0;
    int b_tmax = 0, b_dmax = 0;
};

// Neighbour list of one (destination, source) pair of arrays: entry k of
// destination slot s at nbr[k * stride + s] (k-major, coalesced for
// consecutive destinations), count in cnt[s].  Destinations with more than
// cap neighbours keep the first cap and are completed by a re-traversal.
struct NbrList {
    uint32_t *nbr = nullptr;
    // brick-staged list: entry k of destination d of brick b at
    // nbr16[bdst[b] * cap + k * D_b + d] (an index into the brick's staged
    // sources), count in cnt[bdst[b] + d]
    uint16_t *nbr16 = nullptr;
    bool brick = false;
    int *cnt = nullptr;
    int *maxcnt = nullptr;   // device: largest count of the last list build
    bool own_maxcnt = false; // maxcnt allocated apart (lists past the status block)
    int64_t entries = 0;     // allocated entries
    int64_t stride = 0;
    int64_t stride_cap = 0;  // allocated count slots
    int cap = 0;
    long long build = -1;    // build id the list belongs to
    int seen_max = 0;        // largest count observed (host copy)
};

}  // namespace sphgb

struct sph_step;

struct sph_ctx {
    int dim = 3;
    cudaStream_t stream = 0;
    std::vector<sphgb::ArraySnap> arrays;
    sphgb::Grid grid;
    bool built = false;
    // small device / pinned scratch
    int *d_box = nullptr;               // [6] internal-cell min xyz, max xyz
    unsigned long long *d_hmax = nullptr;
    unsigned *d_err = nullptr;
    // host mirrors written by kernels through mapped page-locked memory (no
    // copy engine: a read-back of the caller's data on a copy stream cannot
    // delay them): box[6], hmax bits (2 words), hmin bits (2 words)
    int *h_box = nullptr;
    int *hd_box = nullptr;              // device address of h_box
    int *scan_tmp = nullptr;
    int64_t scan_tmp_cap = 0;
    double *d_part = nullptr;           // reduction partials
    double *h_red = nullptr;            // pinned
    int64_t *d_cnt = nullptr;           // int64 scratch (mean neighbours)
    int64_t cnt_cap = 0;
    double cell_size_ref = 0;           // reference cell size of the jump check
    long long build_id = 0;             // incremented by every neighbour build
    std::vector<sphgb::NbrList> lists;  // narrays x narrays (dst-major)
    unsigned *d_status = nullptr;       // kStatusWords: error word, displacement, stale, list maxima
    unsigned *h_status = nullptr;       // mapped mirror of d_status
    unsigned *hd_status = nullptr;      // device address of h_status
    // deferred check of a light refresh (sph_ctx_set_deferred): the status
    // of the refresh is read at the next pair pass, which is launched first
    // with gate = &d_status[2] (the pass returns at once when the word is
    // set) and launched again after a full build if it was
    int deferred = 0;
    bool pending = false;               // a refresh whose status is not read yet
    // list entries of this build use code variant 4 (base-5 offsets, 25
    // slot bits): stencil half-width 2 with more than 2^23 source particles
    bool wide_codes = false;
    cudaEvent_t pending_event = nullptr; // recorded after the status copy
    std::vector<sph_array_view> pending_views;
    double pending_cell_size = 0.0, pending_radius_scale = 0.0;
    int pending_subdiv = 1;
    const unsigned *gate = nullptr;     // set while a gated pass is launched
    long long n_deferred = 0, n_deferred_stale = 0;
    // neighbour-list skin as a fraction of the search radius (0 = none)
    double skin_frac = 0.0;
    double build_radius_scale = 0.0;    // parameters of the last full build
    double build_h = 0.0;               // the uniform h of the last full build (0: not uniform)
    int build_subdiv = 0;
    int symmetric = 0;                  // variable-h neighbour relation (next build)
    int periodic = 0;                   // periodic x axis (next build)
    double pxmin = 0.0, pxmax = 0.0;
    long long n_full = 0, n_light = 0;  // full builds / light refreshes
    // brick-staged pair passes (sph_ctx_set_bricks): on by default; ready
    // once the brick tables of the current build are known on the host
    int bricks_on = 1;
    bool bricks_ready = false;
    sphgb::BrickGeom bricks;
    unsigned *d_bstats = nullptr;       // 2 words per array: staged max, destinations max
    unsigned *h_bstats = nullptr;       // mapped mirror
    unsigned *hd_bstats = nullptr;
    long long n_brick_passes = 0;       // pair passes run by the brick kernels
    // step programs (sph_step_*): calls recorded instead of run, and the
    // capture of a recorded step into a CUDA graph (every launch gated on
    // the stale word, no host synchronisation)
    struct sph_step *recording = nullptr;
    bool capturing = false;
    bool capture_failed = false;
    int capture_fail_site = 0;          // where the last capture attempt needed the host
    unsigned capture_stale_bit = 0;     // stale bit of the light refresh being captured
};

namespace sphgb {
// The instances of a batch that share one cell subdivision: their particles
// occupy the sorted slots [s0, s1) (their cells are laid out group by group)
struct BatchGroup {
    int K = 1;
    int64_t s0 = 0, s1 = 0;
};
}  // namespace sphgb

struct sph_batch {
    cudaStream_t stream = nullptr;
    sph_ctx *ctx = nullptr;      // stream + scan scratch for the shared launchers
    sph_array_view view{};
    sph_batch_recipe rec{};
    int ninst = 0;
    std::vector<sphgb::Grid> h_grids;
    sphgb::Grid *d_grids = nullptr;
    double *d_inv_ref = nullptr; // 1 / reference cell size per instance
    int *inst_of = nullptr;      // original particle -> instance
    int *sinst = nullptr;        // sorted slot -> instance
    int64_t total_cells = 0;
    int uniform_h = 1;
    sphgb::ArraySnap snap;
    sphgb::NbrList list;
    double *rate1[6] = {nullptr}, *rate2[6] = {nullptr}, *x0[6] = {nullptr};
    unsigned *d_err = nullptr;
    unsigned long long *d_pairs = nullptr;  // per-instance pair counts
    long long steps_built = 0;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_kernels = 0;       // kernel nodes of one replay
    bool ready = false;
    // per-instance cell subdivision, the groups of equal subdivision and the
    // regions: a particle that leaves its instance's region stops the step
    // (every state-writing launch is gated on the error word), the regions
    // are re-derived from the current extents grown by margin and the step
    // is repeated
    std::vector<int> inst_subdiv;
    std::vector<int> h_uniform_inst;         // 1: the instance's h is uniform
    std::vector<double> inst_cell;           // reference cell size per instance
    std::vector<int64_t> inst_off;           // instance offsets (ninst + 1)
    std::vector<sphgb::BatchGroup> groups;
    double margin = 1.0;
    int64_t cell_cap = 0;                    // allocated cell-table entries
    int64_t *d_off = nullptr;                // instance offsets on the device
    double *d_ibox = nullptr;                // per-instance box (6 doubles)
    unsigned long long *d_steps = nullptr;   // completed steps
    unsigned long long h_steps = 0;
    long long regrids = 0;
};

namespace sphgb {

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
int set_error(int code, const std::string &msg);
int cuda_check(cudaError_t e, const char *what);
#define SPH_CUDA(call)                                          \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return sphgb::cuda_check(e_, #call); \
    } while (0)
#define SPH_LAUNCH_CHECK(what)                                  \
    do {                                                        \
        cudaError_t e_ = cudaGetLastError();                    \
        if (e_ != cudaSuccess) return sphgb::cuda_check(e_, what); \
    } while (0)

int grid_blocks(int64_t n, int threads, int per_sm = 8);

// kernels launched by this library (diagnostic counter, sph_launch_count)
void count_launch(int n = 1);

// launchers implemented in the .cu files
int nnps_build(sph_ctx *ctx, const sph_array_view *arrays, int narrays, double cell_size,
               double radius_scale, int subdiv, int check_jump);
int nnps_update(sph_ctx *ctx, const sph_array_view *arrays, int narrays, double cell_size,
                double radius_scale, int subdiv, int check_jump, int *rebuilt);
int nnps_count(sph_ctx *ctx, int dst, int src, double radius_scale, int64_t *counts);
int nnps_fill(sph_ctx *ctx, int dst, int src, double radius_scale, const int64_t *offsets,
              int64_t *index);
int refresh_state(sph_ctx *ctx, int a, const sph_array_view *view);
// bring the state record st of array a up to date if a light refresh left it
int ensure_state(sph_ctx *ctx, int a);
int selftest_conversions(int64_t n, int64_t *mismatches);
// read the status of a deferred light refresh; *rebuilt: it was stale and a
// full build replaced it (a gated pass launched since then did nothing)
int resolve_pending(sph_ctx *ctx, bool *rebuilt);
inline int resolve_pending(sph_ctx *ctx) {
    bool rebuilt;
    return resolve_pending(ctx, &rebuilt);
}
int launch_adke_smoothing(sph_ctx *ctx, int64_t n, int64_t nreal, const int64_t *tag,
                          const double *rhop, double h0, double k, double eps, double *h);
int launch_adke_conduction(sph_ctx *ctx, int64_t nreal, const int64_t *tag, const double *cs,
                           const double *h, const double *div, double g1, double g2,
                           double *q);
int launch_density(sph_ctx *ctx, int dst, const int *srcs, int nsrc,
                   const sph_density_params *prm, double *rho, double *p, double *cs);
int launch_rates(sph_ctx *ctx, int dst, const sph_source_term *terms, int nterms,
                 const sph_rates_params *prm, double *const *acc, double *const *pos,
                 int accumulate);
int launch_tait(sph_ctx *ctx, int64_t n, const double *rho, const int64_t *tag, double co,
                double ro, double gamma, double *p, double *cs);
int launch_const_rates(sph_ctx *ctx, int kind, int64_t n, const int64_t *tag, const double *g3,
                       const double *u, const double *v, const double *w, int nout,
                       double *const *out);
int launch_integrate(sph_ctx *ctx, int64_t n, const sph_axpy_line *lines, int nlines);
int invariants(sph_ctx *ctx, const sph_array_view *a, double *out);
int build_lists(sph_ctx *ctx, int dst, const int *srcs, int nsrc);
// step programs (program.cu): recording of the calls of one step
int record_update(sph_ctx *ctx, bool build, const sph_array_view *arrays, int narrays,
                  double cell_size, double radius_scale, int subdiv, int check_jump);
int record_density(sph_ctx *ctx, int dst, const int *srcs, int nsrc, const sph_density_params *prm,
                   double *rho, double *p, double *cs);
int record_rates(sph_ctx *ctx, int dst, const sph_source_term *terms, int nterms,
                 const sph_rates_params *prm, double *const *acc, double *const *pos,
                 int accumulate);
int record_tait(sph_ctx *ctx, int64_t n, const double *rho, const int64_t *tag, double co,
                double ro, double gamma, double *p, double *cs);
int record_const(sph_ctx *ctx, int kind, int64_t n, const int64_t *tag, const double *g3,
                 const double *u, const double *v, const double *w, int nout, double *const *out);
int record_integrate(sph_ctx *ctx, int64_t n, const sph_axpy_line *lines, int nlines);
int record_refresh(sph_ctx *ctx, int array, const sph_array_view *view);
// brick-staged pair passes (bricks.cu)
constexpr int kMaxBrickArrays = 16;
void brick_geometry(sph_ctx *ctx);
int brick_tables(sph_ctx *ctx, int a, unsigned *stats);
bool brick_density_eligible(const sph_ctx *ctx, int dst, const int *srcs, int nsrc,
                            const sph_density_params *prm);
bool brick_rates_eligible(const sph_ctx *ctx, int dst, const sph_source_term *terms, int nterms,
                          const sph_rates_params *prm);
int brick_density(sph_ctx *ctx, int dst, int src, NbrList &L, bool build, bool write_out,
                  const sph_density_params *prm, double *rho, double *p, double *cs,
                  float4 *st_out);
int brick_rates(sph_ctx *ctx, int dst, const sph_source_term &term, NbrList &L,
                const sph_rates_params *prm, double *const *acc, double *const *pos,
                int accumulate);
int scan_exclusive(sph_ctx *ctx, int *data, int64_t n);
void launch_counting_sort(cudaStream_t st, int64_t n, int64_t ncells, const int *key, int *cursor,
                          const int *cstart, int *perm);
int batch_setup(sph_batch *b, const sph_array_view *all, const sph_batch_instance *inst,
                int ninst, const sph_batch_recipe *rec);
int batch_build(sph_batch *b, int check_jump);
int batch_density(sph_batch *b);
int batch_rates(sph_batch *b, double *const *acc, double *const *pos);
int batch_step(sph_batch *b, int nsteps, int use_graph);
int batch_pair_counts(sph_batch *b, unsigned long long *out);

// learned momentum closure
int launch_features(sph_ctx *ctx, int dst, int src, const sph_mlp_feature_params *prm,
                    uint16_t *out_bf, float *out_f);
int mlp_grid(int64_t n);
int64_t mlp_backward_scratch(int64_t n);
int mlp_sync(const sph_mlp_model *M, cudaStream_t st);
int mlp_forward(const sph_mlp_model *M, const uint16_t *x, int64_t n, float *y, float *z1,
                float *z2, uint16_t *h1, uint16_t *h2, unsigned *err, cudaStream_t st);
int mlp_backward(const sph_mlp_model *M, const uint16_t *x, const uint16_t *h1, const uint16_t *h2,
                 const float *z1, const float *z2, const float *y, const float *target, int64_t n,
                 float inv_count, float *grad, float *loss, float *scratch, unsigned *err,
                 cudaStream_t st);
int mlp_adam(const sph_mlp_model *M, const float *grad, float *m, float *v, float lr, float beta1,
             float beta2, float eps, int step, cudaStream_t st);
int mlp_apply(int64_t n, const float *y, const int64_t *tag, const double *h, double c0,
              const double *scale, const double *mean, double *const *acc, int accumulate,
              cudaStream_t st);
int mlp_targets(int64_t n, const double *ax, const double *ay, const double *h, double c0,
                const double *mean, const double *inv_std, float *out, cudaStream_t st);
void batch_free(sph_batch *b);
int list_maxima_async(sph_ctx *ctx);
// copy nwords 32-bit words from device memory to a mapped host mirror
// (device address dst) with a one-block kernel on the context's stream
int publish_words(sph_ctx *ctx, const void *src, void *dst, int nwords);
void list_maxima_collect(sph_ctx *ctx);
void free_lists(sph_ctx *ctx);

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------

// Neumaier-compensated FP32 accumulator (sum = hi + lo).
struct CSum {
    float hi, lo;
    __device__ __forceinline__ CSum() : hi(0.f), lo(0.f) {}
    __device__ __forceinline__ void add(float x) {
        float t = hi + x;
        float e = (fabsf(hi) >= fabsf(x)) ? ((hi - t) + x) : ((x - t) + hi);
        hi = t;
        lo += e;
    }
    // merge another compensated sum (error-free TwoSum of the leading parts)
    __device__ __forceinline__ void merge(float ohi, float olo) {
        float s = hi + ohi;
        float bp = s - hi;
        float err = (hi - (s - bp)) + (ohi - bp);
        hi = s;
        lo = lo + olo + err;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
    // the sum rounded to FP32
    __device__ __forceinline__ float fvalue() const { return hi + lo; }
};

// cubic spline normalisation for h = 1 (base/kernels.pyx:437-443)
__device__ __forceinline__ float cubic_fac(int dim, float ih) {
    // 1D: 2/3, 2D: 10/(7 pi), 3D: 1/pi, times h^-dim
    if (dim == 3) return 0.318309886183790672f * ih * ih * ih;
    if (dim == 2) return 0.454728408833986667f * ih * ih;
    return 0.666666666666666667f * ih;
}

// W(q) / fac  (base/kernels.pyx:351-374)
__device__ __forceinline__ float cubic_w(float q) {
    float t = 2.f - q;
    float outer = 0.25f * t * t * t;
    float inner = 1.f - 1.5f * (q * q) * (1.f - 0.5f * q);
    return q > 2.f ? 0.f : (q > 1.f ? outer : inner);
}

// dW/dr / (r fac)  (base/kernels.pyx:376-413); ih = 1/h, rinv = 1/r
__device__ __forceinline__ float cubic_gfac(float q, float ih, float rinv) {
    float t = 2.f - q;
    float outer = -0.75f * t * t * ih * rinv;
    float inner = 3.f * (0.75f * q - 1.f) * ih * ih;
    return q > 2.f ? 0.f : (q >= 1.f ? outer : (q > 1e-14f ? inner : 0.f));
}

// FP64 neighbour test exactly as base/nnps.pyx:337-353 (no FMA contraction):
// d2 = (sx-px)^2 + (sy-py)^2 + (sz-pz)^2 < (radius_scale*h)^2
__device__ __forceinline__ bool exact_within(double sx, double sy, double sz, double px,
                                             double py, double pz, double radius2) {
    double dx = __dsub_rn(sx, px), dy = __dsub_rn(sy, py), dz = __dsub_rn(sz, pz);
    double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return d2 < radius2;
}

__device__ __forceinline__ double ld0(const double *p, int64_t i) { return p ? p[i] : 0.0; }

// Per-source view used by the pair kernels.

struct SrcDev {
    const float4 *velh, *st, *nrm, *tan, *pm;
    const float *scx;
    const int *cstart, *perm;
    const double *x, *y, *z, *h;
    const uint32_t *nbr;   // k-major neighbour list of (dest, this source)
    const int *ncnt;       // neighbour count per dest slot
    uint32_t flags;
    float alpha, beta, eta2, eps, delp;
};

// Neighbour-list entry: source slot j in the low bits, the stencil offset
// of the source's cell in the high BITS bits as three fields of FB bits,
// (dx+K) | (dy+K) << FB | (dz+K) << 2 FB, so the passes that stream a list
// decode the offset with shifts and masks (no table lookup).
template <int K>
struct Code {
    static constexpr int W = 2 * K + 1;
    static constexpr int FB = K == 1 ? 2 : 3;
    static constexpr int BITS = 3 * FB;
    static constexpr int SHIFT = 32 - BITS;
    static constexpr uint32_t JMASK = (1u << SHIFT) - 1u;
    static constexpr uint32_t FMASK = (1u << FB) - 1u;
    // code of a row (dy, dz) with dx = 0; adding dx gives the full code
    __host__ __device__ static constexpr int row(int dy, int dz) {
        return K | ((dy + K) << FB) | ((dz + K) << (2 * FB));
    }
};

// Code variant 4: stencil half-width 2 with the offset in base 5,
// (dx+2) + 5 (dy+2) + 25 (dz+2) (125 values, 7 bits), so the slot keeps 25
// bits (2^25 source particles instead of the 2^23 of three 3-bit fields).
// Linear in dx like the bit fields: a row code plus dx is the full code.
template <>
struct Code<4> {
    static constexpr int BITS = 7;
    static constexpr int SHIFT = 32 - BITS;
    static constexpr uint32_t JMASK = (1u << SHIFT) - 1u;
    __host__ __device__ static constexpr int row(int dy, int dz) {
        return 2 + 5 * (dy + 2) + 25 * (dz + 2);
    }
};

// stencil half-width K of a code variant
template <int KX>
__host__ __device__ constexpr int stencil_k() { return KX == 4 ? 2 : KX; }

// Minus the cell offset (dx, dy, dz) of list entry e, as exact floats: a
// field v becomes 2^23 + v by OR-ing it into the bits of 2^23, and
// (2^23 + K) - (2^23 + v) = -(v - K).
template <int K>
__device__ __forceinline__ float3 neg_cell_offset(uint32_t e) {
    using C = Code<K>;
    const uint32_t c = e >> C::SHIFT;
    constexpr float base = 8388608.f + (float)K;
    return make_float3(base - __uint_as_float((c & C::FMASK) | 0x4B000000u),
                       base - __uint_as_float(((c >> C::FB) & C::FMASK) | 0x4B000000u),
                       base - __uint_as_float(((c >> (2 * C::FB)) & C::FMASK) | 0x4B000000u));
}

// base 5: c / 25 = (c 1311) >> 15 for c < 125 and r / 5 = (r 13) >> 6 for
// r < 25 (exact on those ranges; checked for every value by the tests)
template <>
__device__ __forceinline__ float3 neg_cell_offset<4>(uint32_t e) {
    const uint32_t c = e >> Code<4>::SHIFT;
    const uint32_t z = (c * 1311u) >> 15;
    const uint32_t r = c - 25u * z;
    const uint32_t y = (r * 13u) >> 6;
    const uint32_t x = r - 5u * y;
    constexpr float base = 8388608.f + 2.f;
    return make_float3(base - __uint_as_float(x | 0x4B000000u),
                       base - __uint_as_float(y | 0x4B000000u),
                       base - __uint_as_float(z | 0x4B000000u));
}

// The reverse test of the variable-h relation: destination (original index
// oi, FP64 position dx64..) lies within the radius of source slot j, i.e.
// |x_i - x_j|^2 < (radius_scale h_j)^2.  FP32 outside a +-1e-5 relative band
// around the threshold, the FP64 test of base/nnps.pyx:337-353 inside it.
// in_list: within the list radius of j (radius_scale h_j + skin).
template <class Src>
__device__ __forceinline__ bool reverse_within(const Grid &g, const Src &S, int j, float r2, float rx,
                                               const double *dx64, const double *dy64,
                                               const double *dz64, int oi, bool &in_list) {
    const float rj = (float)g.radius_scale * S.velh[j].w;
    const float rj2 = rj * rj;
    const float rl = rj + g.skin;
    in_list = g.skin > 0.f && r2 < rl * rl * (1.f + 2e-5f);
    if (r2 < rj2 * (1.f - 1e-5f)) return true;
    if (r2 > rj2 * (1.f + 1e-5f)) return false;
    const int oj = S.perm[j];
    const double radius = __dmul_rn(S.h[oj], g.radius_scale);
    const double xi = ld0(dx64, oi);
    return exact_within(xi, ld0(dy64, oi), ld0(dz64, oi), image_x(g, ld0(S.x, oj), xi, rx),
                        ld0(S.y, oj), ld0(S.z, oj), __dmul_rn(radius, radius));
}

// Destination state of one thread (cell-local FP32 offsets, dense cell).
struct DestPos {
    float xi_x, xi_y, xi_z;
    int cx, cy, cz;
    float r2lo, r2hi;   // FP32 accept / reject bands around (radius_scale h)^2
    float r2list;       // list radius (radius_scale h + skin)^2 with margin; 0 = no skin
    double radius2;     // exact FP64 threshold
    int orig;           // original index (FP64 recheck)
};

// Visit every source particle within radius of the destination, in a fixed
// order (stencil rows in (dz, dy) order, ascending sorted slot within a
// row).  Each row is first clipped to the chord of the search sphere: rows
// farther than the radius in (y, z) are skipped and the x extent of the
// others is cut to the cells the sphere reaches, so the loop over one row is
// a single contiguous index range.  fn(j, rx, ry, rz, code, exact) gets
// r = x_dest - x_src in FP32, the stencil offset code and whether the source
// is a neighbour.  The FP32 distance is trusted outside a +-1e-5 relative
// band around the threshold; inside it the FP64 test of base/nnps.pyx:
// 337-353 decides, so the set is exactly the reference's.  With a list skin
// (d.r2list > 0) the sources within the list radius that are not neighbours
// are visited too, with exact = false.  scx[j] holds the source's
// dense-grid x cell.
template <int KX, bool EXT, class Fn>
__device__ __forceinline__ void for_neighbours(const Grid &g, const SrcDev &S, const DestPos &d,
                                               const double *dx64, const double *dy64,
                                               const double *dz64, Fn &&fn) {
    constexpr int K = stencil_k<KX>();
    const float csf = g.cs_f;
    const float inv_cs = 1.f / csf;
    // pruning radius: the accept/recheck threshold plus a relative margin
    // that covers FP32 rounding of the slab distances and cell assignment
    const float R2 = fmaxf(fmaxf(d.r2hi, d.r2list), (EXT && g.symmetric) ? g.reach2 : 0.f) * 1.0002f;
    const float cxf = (float)d.cx;
    const int rowstride_z = g.nx * g.ny;  // < 2^27 cells: 32-bit indices
    const int *cst = S.cstart + g.cell_base;
    for (int dz = -g.kz; dz <= g.kz; ++dz) {
        const float ez = fmaxf(0.f, dz > 0 ? (float)dz * csf - d.xi_z
                                           : (dz < 0 ? d.xi_z - (float)(dz + 1) * csf : 0.f));
        const float ez2 = ez * ez;
        if (ez2 > R2) continue;
        const int zbase = (d.cz + dz) * rowstride_z + d.cx;
        const float bz = d.xi_z - (float)dz * csf;
        for (int dy = -g.ky; dy <= g.ky; ++dy) {
            const float ey = fmaxf(0.f, dy > 0 ? (float)dy * csf - d.xi_y
                                               : (dy < 0 ? d.xi_y - (float)(dy + 1) * csf : 0.f));
            const float rem = R2 - fmaf(ey, ey, ez2);
            if (rem < 0.f) continue;
            // chord half-width with a relative margin (covers the rsqrt error)
            const float half = fmaf(rem * rsqrtf(fmaxf(rem, 1e-30f)), 1.0001f, 1e-5f * csf);
            const int tlo = max(-K, __float2int_rd((d.xi_x - half) * inv_cs));
            const int thi = min(K, __float2int_rd((d.xi_x + half) * inv_cs));
            const int c0 = zbase + (d.cy + dy) * g.nx;
            const float by = d.xi_y - (float)dy * csf;
            const int code_yz = Code<KX>::row(dy, dz);
            // the row's x cells [cx + tlo, cx + thi] (relative): one index
            // range, or on a periodic axis up to three -- the cells past the
            // low / high end wrap to the other end, where the sources' cell
            // index is nx more / less than the unwrapped one (wrap -1 / +1)
            auto visit = [&](int rlo, int rhi, int wrap) {
            const int lo = __ldg(cst + c0 + rlo);
            const int hi = __ldg(cst + c0 + rhi + 1);
            const float wshift = (float)(wrap * g.nx);
            for (int j = lo; j < hi; ++j) {
                const float4 pj = __ldg(S.pm + j);
                const float dxc = (__ldg(S.scx + j) + wshift) - cxf;  // exact: small integers in FP32
                const float rx = fmaf(-dxc, csf, d.xi_x - pj.x);
                const float ry = by - pj.y, rz = bz - pj.z;
                const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                bool hit = r2 < d.r2lo;
                if (!hit && r2 <= d.r2hi) {
                    const int oj = S.perm[j];
                    const double xi = ld0(dx64, d.orig);
                    hit = exact_within(EXT ? image_x(g, ld0(S.x, oj), xi, rx) : ld0(S.x, oj),
                                       ld0(S.y, oj), ld0(S.z, oj), xi, ld0(dy64, d.orig),
                                       ld0(dz64, d.orig), d.radius2);
                }
                bool listed = hit || r2 < d.r2list;
                if (EXT && g.symmetric && !hit && r2 <= g.reach2) {
                    bool in_list;
                    hit = reverse_within(g, S, j, r2, rx, dx64, dy64, dz64, d.orig, in_list);
                    listed = listed || hit || in_list;
                }
                if (listed) fn(j, rx, ry, rz, code_yz + (int)dxc, hit);
            }
            };
            if (!EXT || !g.periodic) {
                visit(tlo, thi, 0);
            } else {
                const int a0 = d.cx + tlo, a1 = d.cx + thi;
                if (a0 < 0) visit(a0 + g.nx - d.cx, min(a1, -1) + g.nx - d.cx, -1);
                visit(max(a0, 0) - d.cx, min(a1, g.nx - 1) - d.cx, 0);
                if (a1 >= g.nx) visit(max(a0, g.nx) - g.nx - d.cx, a1 - g.nx - d.cx, 1);
            }
        }
    }
}

// Dense-grid coordinates of a cell key.
__device__ __forceinline__ void decode_cell(const Grid &g, int key, int &cx, int &cy, int &cz) {
    cx = key % g.nx;
    int rest = key / g.nx;
    cy = rest % g.ny;
    cz = rest / g.ny;
}

}  // namespace sphgb
