/*
 * CPU restatement of the PySPH particle-step hot path -- TEST INFRASTRUCTURE.
 *
 * This file is the checker that the GPU path is compared against.  It is
 * compiled by oracle/__init__.py (gcc, -ffp-contract=off so every product
 * and sum is rounded exactly as the reference's Cython/C++ build on x86-64
 * rounds it) and only tests, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py may load it.  Nothing in the product links it.
 *
 * Everything is FP64.  Each function cites the reference routine it
 * restates (paths relative to the reference's source/pysph/).  Given the same
 * neighbour lists in the same order, the pair sums here reproduce the
 * reference bit for bit; the neighbour search reproduces the reference's
 * neighbour sets exactly.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979311600 /* numpy.pi, base/kernels.pyx:25 */

typedef struct {
    int64_t n;
    const double *x, *y, *z, *u, *v, *w, *m, *h, *rho, *p, *cs;
    const double *nx, *ny, *nz, *tx, *ty, *tz; /* boundary normals/tangents */
    const int64_t *tag;                         /* NULL: all LocalReal      */
} orc_array;

/* ---------------------------------------------------------------------- */
/* cubic spline kernel: base/kernels.pyx:345-449 (fac from _fac(1.0) :73,  */
/* h_dim :47-53)                                                           */
/* ---------------------------------------------------------------------- */

static double cs_fac1(int dim) {
    if (dim == 1) return (2. / 3.) / 1.0;
    if (dim == 2) return 10 / (7 * ORC_PI) / (1.0 * 1.0);
    return 1. / ORC_PI / (1.0 * 1.0 * 1.0);
}

static double h_dim(double h, int dim) {
    if (dim == 1) return 1 / h;
    if (dim == 2) return 1 / (h * h);
    return 1 / (h * h * h);
}

/* kernels.pyx:351-374 -- pa = destination, pb = source */
double orc_cubic_w(int dim, double ax, double ay, double az, double bx, double by,
                   double bz, double h) {
    double rab = sqrt((ax - bx) * (ax - bx) + (ay - by) * (ay - by) + (az - bz) * (az - bz));
    double q = rab / h;
    double val;
    double fac = h_dim(h, dim) * cs_fac1(dim);
    if (q > 2.0)
        val = 0.0;
    else if (q > 1.0)
        val = 0.25 * (2 - q) * (2 - q) * (2 - q);
    else
        val = 1 - 1.5 * (q * q) * (1 - 0.5 * q);
    return val * fac;
}

/* kernels.pyx:376-413 */
void orc_cubic_grad(int dim, double ax, double ay, double az, double bx, double by,
                    double bz, double h, double *g) {
    double rab = sqrt((ax - bx) * (ax - bx) + (ay - by) * (ay - by) + (az - bz) * (az - bz));
    double q = rab / h;
    double val = 0.0;
    double fac = h_dim(h, dim) * cs_fac1(dim);
    double rx = ax - bx, ry = ay - by, rz = az - bz;
    if (q > 2.0) {
    } else if (q >= 1.0) {
        val = -0.75 * (2 - q) * (2 - q) / (h * rab);
    } else if (q > 1e-14) {
        val = 3.0 * (0.75 * q - 1) / (h * h);
    }
    g[0] = rx * (val * fac);
    g[1] = ry * (val * fac);
    g[2] = rz * (val * fac);
}

static inline double get0(const double *a, int64_t i) { return a ? a[i] : 0.0; }

/* ---------------------------------------------------------------------- */
/* neighbour search: cell binning base/cell.pyx:42-82 (floor(x/cell_size)),*/
/* stencil :93-116 / :1106-1142 (distance = ceil(radius/cell_size)),       */
/* distance test base/nnps.pyx:271-356 (d2 = |src-dst|^2 < radius^2, with  */
/* radius = radius_scale * h_dst, :525-559), self moved last :596-620.      */
/* Lists are returned in ascending source index, then (src == dst) the      */
/* destination swapped with the last entry, as nnps.pyx:609-616 does.       */
/* ---------------------------------------------------------------------- */

typedef struct { int64_t cx, cy, cz; int64_t idx; } cell_rec;

static int cmp_cell(const void *a, const void *b) {
    const cell_rec *p = (const cell_rec *)a, *q = (const cell_rec *)b;
    if (p->cz != q->cz) return p->cz < q->cz ? -1 : 1;
    if (p->cy != q->cy) return p->cy < q->cy ? -1 : 1;
    if (p->cx != q->cx) return p->cx < q->cx ? -1 : 1;
    return p->idx < q->idx ? -1 : (p->idx > q->idx);
}

static int64_t lower_bound(const cell_rec *r, int64_t n, int64_t cx, int64_t cy, int64_t cz) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        cell_rec k = {cx, cy, cz, -1};
        if (cmp_cell(&r[mid], &k) < 0) lo = mid + 1; else hi = mid;
    }
    return lo;
}

static int cmp_i64(const void *a, const void *b) {
    int64_t p = *(const int64_t *)a, q = *(const int64_t *)b;
    return p < q ? -1 : (p > q);
}

/* Pass 1 (index == NULL): counts into offsets[1..n]; returns total.
 * Pass 2: fills index given prefix offsets.
 * symmetric = 0: j is a neighbour of i when |x_j - x_i|^2 < (radius_scale h_i)^2
 *   (FixedDestNbrParticleLocator, base/nnps.pyx:271-356, 525-620);
 * symmetric = 1: also when |x_i - x_j|^2 < (radius_scale h_j)^2, the union
 *   VarHNbrParticleLocator builds from its reversed locator (base/nnps.pyx:
 *   654-749).                                                             */
/* splitmix64 finaliser: an order-independent digest of a neighbour set is
 * the wrap-around sum of mix(j) over its source indices j. */
static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* digest (pass 1 only, may be NULL): per destination, the sum of mix64(j)
 * over its neighbours -- the set without storing it. */
static int64_t neighbors_impl(const orc_array *dst, const orc_array *src, double cell_size,
                              double radius_scale, int same, int symmetric, int64_t *offsets,
                              int64_t *index, uint64_t *digest) {
    int64_t ns = src->n, nd = dst->n;
    double hmax_src = 0.0;
    for (int64_t j = 0; j < ns; ++j)
        if (src->h[j] > hmax_src) hmax_src = src->h[j];
    cell_rec *recs = (cell_rec *)malloc(sizeof(cell_rec) * (ns > 0 ? ns : 1));
    for (int64_t j = 0; j < ns; ++j) {
        recs[j].cx = (int64_t)(int)floor(get0(src->x, j) / cell_size);
        recs[j].cy = (int64_t)(int)floor(get0(src->y, j) / cell_size);
        recs[j].cz = (int64_t)(int)floor(get0(src->z, j) / cell_size);
        recs[j].idx = j;
    }
    qsort(recs, ns, sizeof(cell_rec), cmp_cell);
    int64_t total = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : total)
    for (int64_t i = 0; i < nd; ++i) {
        double px = get0(dst->x, i), py = get0(dst->y, i), pz = get0(dst->z, i);
        double radius = dst->h[i] * radius_scale;
        double radius2 = radius * radius;
        double reach = radius;
        if (symmetric && hmax_src * radius_scale > reach) reach = hmax_src * radius_scale;
        int64_t d = (int64_t)(int)ceil(reach / cell_size);
        int64_t cx = (int)floor(px / cell_size), cy = (int)floor(py / cell_size),
                cz = (int)floor(pz / cell_size);
        int64_t cnt = 0;
        uint64_t dig = 0;
        int64_t base = index ? offsets[i] : 0;
        for (int64_t a = -d; a <= d; ++a)
            for (int64_t b = -d; b <= d; ++b)
                for (int64_t c = -d; c <= d; ++c) {
                    int64_t k = lower_bound(recs, ns, cx + a, cy + b, cz + c);
                    for (; k < ns && recs[k].cx == cx + a && recs[k].cy == cy + b &&
                           recs[k].cz == cz + c;
                         ++k) {
                        int64_t j = recs[k].idx;
                        double sx = get0(src->x, j), sy = get0(src->y, j), sz = get0(src->z, j);
                        double d2 = ((sx - px) * (sx - px) + (sy - py) * (sy - py) +
                                     (sz - pz) * (sz - pz));
                        int hit = d2 < radius2;
                        if (!hit && symmetric) {
                            double rj = src->h[j] * radius_scale;
                            double e2 = ((px - sx) * (px - sx) + (py - sy) * (py - sy) +
                                         (pz - sz) * (pz - sz));
                            hit = e2 < rj * rj;
                        }
                        if (hit) {
                            if (index) index[base + cnt] = j;
                            if (digest) dig += mix64((uint64_t)j);
                            ++cnt;
                        }
                    }
                }
        if (index) {
            qsort(index + base, cnt, sizeof(int64_t), cmp_i64);
            if (same) {
                for (int64_t t = 0; t + 1 < cnt; ++t)
                    if (index[base + t] == i) {
                        index[base + t] = index[base + cnt - 1];
                        index[base + cnt - 1] = i;
                        break;
                    }
            }
        } else {
            offsets[i + 1] = cnt;
            if (digest) digest[i] = dig;
        }
        total += cnt;
    }
    free(recs);
    return total;
}

int64_t orc_neighbors(const orc_array *dst, const orc_array *src, double cell_size,
                      double radius_scale, int same, int64_t *offsets, int64_t *index) {
    return neighbors_impl(dst, src, cell_size, radius_scale, same, 0, offsets, index, NULL);
}

int64_t orc_neighbors_varh(const orc_array *dst, const orc_array *src, double cell_size,
                           double radius_scale, int same, int64_t *offsets, int64_t *index) {
    return neighbors_impl(dst, src, cell_size, radius_scale, same, 1, offsets, index, NULL);
}

/* Neighbour counts (counts[i + 1], as pass 1 of orc_neighbors) and set
 * digests (digest[i]) of every destination, in memory linear in the
 * particle count: for sets too large to hold as lists. */
int64_t orc_neighbor_digest(const orc_array *dst, const orc_array *src, double cell_size,
                            double radius_scale, int64_t *counts, uint64_t *digest) {
    return neighbors_impl(dst, src, cell_size, radius_scale, 0, 0, counts, NULL, digest);
}

/* ---------------------------------------------------------------------- */
/* SPH functions.  Each adds its per-destination sum into out[] for        */
/* LocalReal destinations and writes 0 otherwise (sph/sph_func.pyx:199-234)*/
/* ---------------------------------------------------------------------- */

#define LOCAL_REAL 0

static inline int is_real(const orc_array *a, int64_t i) {
    return a->tag == NULL || a->tag[i] == LOCAL_REAL;
}

/* SPHRho: sph/funcs/density_funcs.pyx:38-74 (hks=False) */
void orc_sph_rho(const orc_array *d, const orc_array *s, const int64_t *off,
                 const int64_t *idx, int dim, double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) { out[i] = 0; continue; }
        double nr = 0.0;
        for (int64_t k = off[i]; k < off[i + 1]; ++k) {
            int64_t j = idx[k];
            double hab = 0.5 * (d->h[i] + s->h[j]);
            double w = orc_cubic_w(dim, get0(d->x, i), get0(d->y, i), get0(d->z, i),
                                   get0(s->x, j), get0(s->y, j), get0(s->z, j), hab);
            nr += w * s->m[j];
        }
        out[i] += nr;
    }
}

/* TaitEquation: sph/funcs/eos_funcs.pyx:81-116 */
void orc_tait(const orc_array *d, double co, double ro, double gamma, double *p_out,
              double *cs_out) {
    double B = co * co * ro / gamma;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) { p_out[i] = 0; cs_out[i] = 0; continue; }
        double rhoa = d->rho[i];
        double ratio = rhoa / ro;
        double gamma2 = 0.5 * (gamma - 1.0);
        double tmp = pow(ratio, gamma);
        p_out[i] += (tmp - 1.0) * B;
        cs_out[i] += pow(ratio, gamma2) * co;
    }
}

/* SPHPressureGradient: sph/funcs/pressure_funcs.pyx:40-91 */
void orc_pgrad(const orc_array *d, const orc_array *s, const int64_t *off,
               const int64_t *idx, int dim, int nout, double *o0, double *o1, double *o2) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) {
            o0[i] = 0; if (nout > 1) o1[i] = 0; if (nout > 2) o2[i] = 0;
            continue;
        }
        double nr[3] = {0, 0, 0};
        for (int64_t k = off[i]; k < off[i + 1]; ++k) {
            int64_t j = idx[k];
            double mb = s->m[j];
            double rhoa = d->rho[i], rhob = s->rho[j];
            double pa = d->p[i], pb = s->p[j];
            double h = 0.5 * (d->h[i] + s->h[j]);
            double temp = (pa / (rhoa * rhoa) + pb / (rhob * rhob));
            temp *= -mb;
            double g[3];
            orc_cubic_grad(dim, get0(d->x, i), get0(d->y, i), get0(d->z, i), get0(s->x, j),
                           get0(s->y, j), get0(s->z, j), h, g);
            nr[0] += temp * g[0];
            nr[1] += temp * g[1];
            nr[2] += temp * g[2];
        }
        o0[i] += nr[0];
        if (nout > 1) o1[i] += nr[1];
        if (nout > 2) o2[i] += nr[2];
    }
}

/* MonaghanArtificialVsicosity: sph/funcs/viscosity_funcs.pyx:41-124.
 * The reference never stores eta (:21-34), so callers pass eta = 0.       */
void orc_avisc(const orc_array *d, const orc_array *s, const int64_t *off,
               const int64_t *idx, int dim, double alpha, double beta, double eta,
               double *o0, double *o1, double *o2) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) { o0[i] = o1[i] = o2[i] = 0; continue; }
        double nr[3] = {0, 0, 0};
        for (int64_t k = off[i]; k < off[i + 1]; ++k) {
            int64_t j = idx[k];
            double ha = d->h[i], hb = s->h[j];
            double hab = 0.5 * (ha + hb);
            double rx = get0(d->x, i) - get0(s->x, j), ry = get0(d->y, i) - get0(s->y, j),
                   rz = get0(d->z, i) - get0(s->z, j);
            double vx = get0(d->u, i) - get0(s->u, j), vy = get0(d->v, i) - get0(s->v, j),
                   vz = get0(d->w, i) - get0(s->w, j);
            double dot = vx * rx + vy * ry + vz * rz;
            double rhoa = d->rho[i], rhob = s->rho[j];
            double mb = s->m[j];
            double piab = 0;
            if (dot < 0) {
                double cab = 0.5 * (d->cs[i] + s->cs[j]);
                double rhoab = 0.5 * (rhoa + rhob);
                double mu = hab * dot;
                mu /= ((rx * rx + ry * ry + rz * rz) + eta * eta * hab * hab);
                piab = -alpha * cab * mu + beta * mu * mu;
                piab /= rhoab;
            }
            double tmp = piab;
            tmp *= -mb;
            double g[3];
            orc_cubic_grad(dim, get0(d->x, i), get0(d->y, i), get0(d->z, i), get0(s->x, j),
                           get0(s->y, j), get0(s->z, j), hab, g);
            nr[0] += tmp * g[0];
            nr[1] += tmp * g[1];
            nr[2] += tmp * g[2];
        }
        o0[i] += nr[0]; o1[i] += nr[1]; o2[i] += nr[2];
    }
}

/* MomentumEquation: sph/funcs/pressure_funcs.pyx:106-252 -- pressure
 * gradient and Monaghan viscosity in one pair term, eta stored (default
 * 0.1), hks off; num_outputs = dim.                                       */
void orc_momentum(const orc_array *d, const orc_array *s, const int64_t *off,
                  const int64_t *idx, int dim, double alpha, double beta, double eta,
                  int nout, double *o0, double *o1, double *o2) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) {
            o0[i] = 0; if (nout > 1) o1[i] = 0; if (nout > 2) o2[i] = 0;
            continue;
        }
        double nr[3] = {0, 0, 0};
        for (int64_t k = off[i]; k < off[i + 1]; ++k) {
            int64_t j = idx[k];
            double ha = d->h[i], hb = s->h[j];
            double hab = 0.5 * (ha + hb);
            double rx = get0(d->x, i) - get0(s->x, j), ry = get0(d->y, i) - get0(s->y, j),
                   rz = get0(d->z, i) - get0(s->z, j);
            double vx = get0(d->u, i) - get0(s->u, j), vy = get0(d->v, i) - get0(s->v, j),
                   vz = get0(d->w, i) - get0(s->w, j);
            double dot = vx * rx + vy * ry + vz * rz;
            double pa = d->p[i], rhoa = d->rho[i];
            double pb = s->p[j], rhob = s->rho[j], mb = s->m[j];
            double tmp = pa / (rhoa * rhoa) + pb / (rhob * rhob);
            double piab = 0;
            if (dot < 0) {
                double cab = 0.5 * (d->cs[i] + s->cs[j]);
                double rhoab = 0.5 * (rhoa + rhob);
                double mu = hab * dot;
                mu /= ((rx * rx + ry * ry + rz * rz) + eta * eta * hab * hab);
                piab = -alpha * cab * mu + beta * mu * mu;
                piab /= rhoab;
            }
            tmp += piab;
            tmp *= -mb;
            double g[3];
            orc_cubic_grad(dim, get0(d->x, i), get0(d->y, i), get0(d->z, i), get0(s->x, j),
                           get0(s->y, j), get0(s->z, j), hab, g);
            nr[0] += tmp * g[0];
            nr[1] += tmp * g[1];
            nr[2] += tmp * g[2];
        }
        o0[i] += nr[0];
        if (nout > 1) o1[i] += nr[1];
        if (nout > 2) o2[i] += nr[2];
    }
}

/* SPHDensityRate: sph/funcs/density_funcs.pyx:89-158 -- drho_a +=
 * m_b (v_a - v_b) . grad W(r_ab, hab), hks off.                           */
void orc_drho(const orc_array *d, const orc_array *s, const int64_t *off, const int64_t *idx,
              int dim, double *o0) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) { o0[i] = 0; continue; }
        double nr = 0;
        for (int64_t k = off[i]; k < off[i + 1]; ++k) {
            int64_t j = idx[k];
            double hab = 0.5 * (d->h[i] + s->h[j]);
            double vx = get0(d->u, i) - get0(s->u, j), vy = get0(d->v, i) - get0(s->v, j),
                   vz = get0(d->w, i) - get0(s->w, j);
            double g[3];
            orc_cubic_grad(dim, get0(d->x, i), get0(d->y, i), get0(d->z, i), get0(s->x, j),
                           get0(s->y, j), get0(s->z, j), hab, g);
            nr += (vx * g[0] + vy * g[1] + vz * g[2]) * s->m[j];
        }
        o0[i] += nr;
    }
}

/* ADKEPilotRho: sph/funcs/adke_funcs.pyx:41-73 -- rhop_a += m_b W(r_ab, h0)
 * over the neighbours of the destination's own radius (CSPH, no correction) */
void orc_pilot_rho(const orc_array *d, const orc_array *s, const int64_t *off,
                   const int64_t *idx, int dim, double h0, double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) { out[i] = 0; continue; }
        double nr = 0.0;
        for (int64_t k = off[i]; k < off[i + 1]; ++k) {
            int64_t j = idx[k];
            double w = orc_cubic_w(dim, get0(d->x, i), get0(d->y, i), get0(d->z, i),
                                   get0(s->x, j), get0(s->y, j), get0(s->z, j), h0);
            nr += w * s->m[j];
        }
        out[i] += nr;
    }
}

/* SPHVelocityDivergence: sph/funcs/adke_funcs.pyx:175-226 (hks off) --
 * div_a += (1/rho_a) m_b (v_b - v_a) . grad W(r_ab, (h_a + h_b)/2)          */
void orc_vdiv(const orc_array *d, const orc_array *s, const int64_t *off, const int64_t *idx,
              int dim, double *o0) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) { o0[i] = 0; continue; }
        double nr = 0;
        for (int64_t k = off[i]; k < off[i + 1]; ++k) {
            int64_t j = idx[k];
            double hab = 0.5 * (d->h[i] + s->h[j]);
            double vx = get0(s->u, j) - get0(d->u, i), vy = get0(s->v, j) - get0(d->v, i),
                   vz = get0(s->w, j) - get0(d->w, i);
            double g[3];
            orc_cubic_grad(dim, get0(d->x, i), get0(d->y, i), get0(d->z, i), get0(s->x, j),
                           get0(s->y, j), get0(s->z, j), hab, g);
            nr += (1.0 / d->rho[i]) * s->m[j] * (g[0] * vx + g[1] * vy + g[2] * vz);
        }
        o0[i] += nr;
    }
}

/* XSPHCorrection: sph/funcs/xsph_funcs.pyx:31-88 (CSPH, no correction) */
void orc_xsph(const orc_array *d, const orc_array *s, const int64_t *off,
              const int64_t *idx, int dim, double eps, int nout, double *o0, double *o1,
              double *o2) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) {
            o0[i] = 0; if (nout > 1) o1[i] = 0; if (nout > 2) o2[i] = 0;
            continue;
        }
        double nr[3] = {0, 0, 0};
        for (int64_t k = off[i]; k < off[i + 1]; ++k) {
            int64_t j = idx[k];
            double hab = 0.5 * (d->h[i] + s->h[j]);
            double rhoab = 0.5 * (s->rho[j] + d->rho[i]);
            double vbx = get0(s->u, j) - get0(d->u, i), vby = get0(s->v, j) - get0(d->v, i),
                   vbz = get0(s->w, j) - get0(d->w, i);
            double mb = s->m[j];
            double w = orc_cubic_w(dim, get0(d->x, i), get0(d->y, i), get0(d->z, i),
                                   get0(s->x, j), get0(s->y, j), get0(s->z, j), hab);
            double temp = mb * w / rhoab;
            nr[0] += temp * vbx * eps;
            nr[1] += temp * vby * eps;
            nr[2] += temp * vbz * eps;
        }
        o0[i] += nr[0];
        if (nout > 1) o1[i] += nr[1];
        if (nout > 2) o2[i] += nr[2];
    }
}

/* MonaghanBoundaryForce: sph/funcs/boundary_funcs.pyx:54-110 */
void orc_bforce(const orc_array *d, const orc_array *s, const int64_t *off,
                const int64_t *idx, double delp, double *o0, double *o1, double *o2) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) { o0[i] = o1[i] = o2[i] = 0; continue; }
        double nr[3] = {0, 0, 0};
        for (int64_t k = off[i]; k < off[i + 1]; ++k) {
            int64_t j = idx[k];
            double h = d->h[i];
            double ma = d->m[i], mb = s->m[j];
            double nx = get0(s->nx, j), ny = get0(s->ny, j), nz = get0(s->nz, j);
            double tx = get0(s->tx, j), ty = get0(s->ty, j), tz = get0(s->tz, j);
            double cs = d->cs[i];
            double rx = get0(d->x, i) - get0(s->x, j), ry = get0(d->y, i) - get0(s->y, j),
                   rz = get0(d->z, i) - get0(s->z, j);
            double x = rx * tx + ry * ty + rz * tz;
            double y = rx * nx + ry * ny + rz * nz;
            double force = 0.0, nforce, beta, tforce;
            double q = y / h;
            if (0 <= fabs(x) && fabs(x) <= delp) {
                beta = 0.02 * cs * cs / y;
                tforce = 1.0 - fabs(x) / delp;
                if (0 < q && q <= 2.0 / 3.0)
                    nforce = 2.0 / 3.0;
                else if (2.0 / 3.0 < q && q <= 1.0)
                    nforce = 2 * q * (1.0 - 0.75 * q);
                else if (1.0 < q && q <= 2.0)
                    nforce = 0.5 * (2 - q) * (2 - q);
                else
                    nforce = 0.0;
                force = (mb / (ma + mb)) * nforce * tforce * beta;
            }
            nr[0] += force * nx;
            nr[1] += force * ny;
            nr[2] += force * nz;
        }
        o0[i] += nr[0]; o1[i] += nr[1]; o2[i] += nr[2];
    }
}

/* GravityForce: sph/funcs/external_force.pyx:39-45; PositionStepping:
 * sph/funcs/position_funcs.pyx:32-60 (k = velocity).                     */
void orc_const3(const orc_array *d, double gx, double gy, double gz, int nout, double *o0,
                double *o1, double *o2) {
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) {
            o0[i] = 0; if (nout > 1) o1[i] = 0; if (nout > 2) o2[i] = 0;
            continue;
        }
        o0[i] += gx; if (nout > 1) o1[i] += gy; if (nout > 2) o2[i] += gz;
    }
}

void orc_position_stepping(const orc_array *d, int nout, double *o0, double *o1, double *o2) {
    for (int64_t i = 0; i < d->n; ++i) {
        if (!is_real(d, i)) {
            o0[i] = 0; if (nout > 1) o1[i] = 0; if (nout > 2) o2[i] = 0;
            continue;
        }
        o0[i] += get0(d->u, i);
        if (nout > 1) o1[i] += get0(d->v, i);
        if (nout > 2) o2[i] += get0(d->w, i);
    }
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
