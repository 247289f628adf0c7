/*
 * sph_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * FP64 CPU restatement of pyticles' SPH step, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline / reference legs to
 * compare results against.  Nothing in pyticles_gb300/ links or calls it.
 *
 * Parity pinning: tests/test_oracle_golden.py checks this file against golden
 * vectors in tests/golden/ that tests/golden/make_golden.py produced by
 * running the reference's own pure-Python functions (spkernel.lucy_kernel,
 * gauss_kernel, debrun_kernel, spdensity.sum_density, properties.vdw*,
 * forces.SpamForce / CohesiveSpamForce, neighbour_list.VerletList.build,
 * NeighbourList.separations, integrator.imp_euler/euler/rk4,
 * box.PeriodicBox.apply, SmoothParticleSystem.update).  The artificial
 * viscosity, the heat-flux vector and the cubic-spline kernel have no source
 * in the reference (their Fortran modules are absent), so those terms are
 * parity-unpinned restatements of the published formulas named below.
 *
 * Semantics (reference file:line in andrewcharles/pyticles):
 *  pair set   i<j, dr = r_j - r_i, one minimum-image shift per axis with
 *             strict > / < against box/2 (neighbour_list.py:105-123), rsq =
 *             dx*dx + dy*dy (+ dz*dz) summed left to right, kept when
 *             rsq < cutoff^2 + tolerance^2 (neighbour_list.py:168-189).
 *  kernels    Lucy (spkernel.py:86-118), Gaussian (spkernel.py:39-52, gradient
 *             sign flipped to Lucy's convention dwdx = dW/dr (r_j-r_i)/r),
 *             Debrun (spkernel.py:120-153, constants as written there), M4
 *             cubic spline (Monaghan & Lattanzio 1985, support 2h).
 *  density    rho_i = W(0,h) + sum_j m_j W(r_ij,h); self term without m_i
 *             (properties.py:77-91, spdensity.py:40-56); rho_lr the same with
 *             the long smoothing length.
 *  EOS        T = (u + a rho)/k_B clamped at 0 (properties.py:48-49,
 *             spam_complete_force.py:134,151-152); p = rho k_B T/(1 - b rho)
 *             and pco = -a rho_lr^2 (properties.py:38-41, f_properties.py:119).
 *  forces     per pair ps = p_i/rho_i^2 + p_j/rho_j^2 (+ Pi_ij), a = ps dwdx,
 *             vdot_i += a, vdot_j -= a (no mass factor), du = a.dv/2,
 *             udot_i += du m_j, udot_j += du m_i (forces.py:338-405,
 *             c_forces.pyx:96-111,163-178); cohesive term with pco, rho_lr and
 *             the long-h gradient.
 *  viscosity  Monaghan (1992, ARA&A 30:543) Pi_ij = (-alpha c mu + beta mu^2)
 *             / rho_bar when v_ij.r_ij < 0, mu = h v_ij.r_ij/(r^2 + eps h^2),
 *             on the short smoothing length; added to ps.  (unpinned)
 *  heat flux  q_i = kappa sum_j (m_j/rho_j)(T_j - T_i) dwdx_ij  (Fourier,
 *             -kappa grad T with grad_i W = -dwdx; f_properties.py:129-130);
 *             udot_i -= m_j (q_i/rho_i^2 + q_j/rho_j^2).dwdx,
 *             udot_j += m_i (...) (c_forces.pyx:224-237).  (q unpinned)
 *  integrator imp_euler / euler / rk4 on (r, v, u) with rates (v, vdot, udot)
 *             (integrator.py:14-103); c = f*dt, x = x0 + c, ...
 *  box        teleport wrap: r > L -> 0, r < 0 -> L per axis (box.py:33-47).
 *  collisions after each evaluation (forces after SpamComplete in p.forces):
 *             the pair list in (i, j) order, pairs with rij^2 <= cutoff^2
 *             (forces.py:38-42) that are not separating trade the velocity
 *             components along dr, scaled by the mass ratio, sequentially
 *             (CollisionForce forces.py:87-156; FortranCollisionForce's absent
 *             collide3d restated the same way, forces.py:454-474);
 *             CollisionForce3d also pushes the pair apart to cutoff + 0.01
 *             (forces.py:158-243).  In a step, the extra first evaluation of
 *             update() (particles.py:480) leaves its collisions behind and the
 *             first evaluation's collided velocities are x_start's
 *             (integrator.py:44-59).
 *  thermostat T <- T_last * target/mean(T_last); u <- k_B T - a rho, with
 *             T_last the temperature of the step's last evaluation and rho
 *             the start-of-step density (particles.py:450-457, 513-526;
 *             get_vdw_u restated as properties.vdw_energy, properties.py:44-46).
 *
 * Compile with -ffp-contract=off so the FP64 pair test matches the
 * reference's separately rounded products and sums.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/sph.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct {
    int dim;
    int nc[3];
    double edge[3];
    int64_t ncell;
    int64_t *start; /* ncell + 1 */
    int64_t *idx;   /* n */
} grid_t;

static int g_threads = 0;

/* FP32 pair geometry (orc_set_geometry32): every pair's separation vector
 * and distance are replaced by the FP32 numbers nearest to them before any
 * kernel or force term uses them; the pair set and everything else stay
 * FP64.  The change this makes to a result is the error floor of any
 * evaluation that carries pair geometry in FP32, however accurate its other
 * arithmetic: the reference against which the mixed-precision passes are
 * held on near-lattice systems whose pair forces cancel. */
static int g_geom32 = 0;

void orc_set_geometry32(int on) { g_geom32 = on ? 1 : 0; }

static inline void geometry32(int dim, double *dr, double *rsq) {
    for (int a = 0; a < dim; ++a) dr[a] = (double)(float)dr[a];
    double r = (double)(float)sqrt(*rsq);
    *rsq = r * r; /* exact: sqrt(*rsq) is then r again */
}

void orc_set_threads(int n) { g_threads = n; }

int orc_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- kernels (W and the Lucy-convention gradient factor) -------------- */

/* Returns W(r,h) and g such that dwdx = g * (r_j - r_i); g = 0 at r == 0. */
static void kern(int type, int dim, double r, double h, double *w, double *g) {
    *w = 0.0;
    *g = 0.0;
    if (type == SPH_KERNEL_LUCY) {
        double q;
        if (dim == 1) q = 5. / (4. * h);
        else if (dim == 2) q = 5. / (M_PI * h * h);
        else q = 105. / (M_PI * 16. * (h * h * h));
        if (r < h) {
            double s = 1. - r / h;
            *w = q * (1 + 3. * r / h) * (s * s * s);
            if (r != 0.0) {
                double h2 = h * h, h3 = h2 * h, h4 = h3 * h;
                *g = q * ((-12. / h4) * (r * r * r) + (24. / h3) * (r * r) - (12. * r / h2)) / r;
            }
        }
    } else if (type == SPH_KERNEL_GAUSSIAN) {
        double q = r / h;
        double factor = 1.e0 / (pow(h, dim) * pow(M_PI, dim / 2.));
        *w = factor * exp(-q * q);
        *g = -2.0 * (*w) / (h * h); /* spkernel.py:51 has the opposite sign */
    } else if (type == SPH_KERNEL_DEBRUN) {
        if (r < h) {
            double q;
            double h2 = h * h, h4 = h2 * h2, h6 = h4 * h2;
            if (dim == 1) q = (1.0 / ((-7. * h4 / 4) + 2 * h4)) / 2;
            else if (dim == 2) q = 10.0 / (M_PI * h6);
            else q = 15.0 / (M_PI * h6);
            double s = h - r;
            *w = q * (s * s * s);
            if (r != 0.0) *g = q * (-3.0 * h2 + 6.0 * h * r - 3.0 * (r * r)) / r;
        }
    } else if (type == SPH_KERNEL_CUBIC) {
        double sig;
        if (dim == 1) sig = 2.0 / (3.0 * h);
        else if (dim == 2) sig = 10.0 / (7.0 * M_PI * h * h);
        else sig = 1.0 / (M_PI * h * h * h);
        double q = r / h;
        if (q < 1.0) {
            *w = sig * (1.0 - 1.5 * q * q + 0.75 * q * q * q);
            *g = sig * (-3.0 + 2.25 * q) / (h * h);
        } else if (q < 2.0) {
            double s = 2.0 - q;
            *w = sig * 0.25 * s * s * s;
            *g = -0.75 * sig * s * s / (h * r);
        }
    }
}

/* ---- pair geometry exactly as neighbour_list.py ------------------------ */

static inline double min_image(double d, double L) {
    if (d > L / 2.) d = d - L;
    if (d < -L / 2.) d = d + L;
    return d;
}

/* dr = r_j - r_i, minimum-imaged; returns rsq summed left to right. */
static inline double pair_rsq(const sph_params *p, const double *ri, const double *rj,
                              double *dr) {
    int d = p->dim;
    double rsq = 0.0;
    for (int a = 0; a < d; ++a) {
        double x = rj[a] - ri[a];
        x = min_image(x, p->box[a]);
        dr[a] = x;
        double sq = x * x;
        rsq = (a == 0) ? sq : rsq + sq;
    }
    return rsq;
}

static double pair_threshold(const sph_params *p) {
    double csq = p->cutoff * p->cutoff;
    double tsq = p->tolerance * p->tolerance;
    return csq + tsq;
}

/* ---- cell grid --------------------------------------------------------- */

static int grid_build(const sph_params *p, int64_t n, const double *r, grid_t *g) {
    int d = p->dim;
    double rc = sqrt(pair_threshold(p)) * (1.0 + 1e-9);
    g->dim = d;
    g->ncell = 1;
    for (int a = 0; a < 3; ++a) {
        if (a >= d) {
            g->nc[a] = 1;
            g->edge[a] = 1.0;
            continue;
        }
        double q = floor(p->box[a] / rc);
        int nc = q > 1e6 ? 1000000 : (int)q;
        if (nc < 3) nc = 1;
        g->nc[a] = nc;
    }
    /* a sparse system in a large box: coarser cells, at most 8 per particle
     * (at least 2^16) */
    int64_t limit = 8 * n > (1 << 16) ? 8 * n : (1 << 16);
    for (;;) {
        int64_t total = (int64_t)g->nc[0] * g->nc[1] * g->nc[2];
        if (total <= limit) break;
        int a = 0;
        for (int b = 1; b < d; ++b)
            if (g->nc[b] > g->nc[a]) a = b;
        int nc = (int)(g->nc[a] * 0.9);
        g->nc[a] = nc < 3 ? 1 : nc;
    }
    for (int a = 0; a < 3; ++a) {
        g->edge[a] = a < d ? p->box[a] / g->nc[a] : 1.0;
        g->ncell *= g->nc[a];
    }
    g->start = (int64_t *)calloc((size_t)g->ncell + 1, sizeof(int64_t));
    g->idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int64_t *cell = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    if (!g->start || !g->idx || !cell) {
        free(g->start);
        free(g->idx);
        free(cell);
        return SPH_ENOMEM;
    }
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        for (int a = d - 1; a >= 0; --a) {
            double L = p->box[a];
            double x = r[i * d + a];
            x = x - L * floor(x / L);
            int ci = (int)(x / g->edge[a]);
            if (ci < 0) ci = 0;
            if (ci >= g->nc[a]) ci = g->nc[a] - 1;
            c = c * g->nc[a] + ci;
        }
        cell[i] = c;
        g->start[c + 1]++;
    }
    for (int64_t c = 0; c < g->ncell; ++c) g->start[c + 1] += g->start[c];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)g->ncell);
    memcpy(fill, g->start, sizeof(int64_t) * (size_t)g->ncell);
    for (int64_t i = 0; i < n; ++i) g->idx[fill[cell[i]]++] = i;
    free(fill);
    free(cell);
    return SPH_OK;
}

static void grid_free(grid_t *g) {
    free(g->start);
    free(g->idx);
    g->start = g->idx = NULL;
}

/* Neighbour cells of particle i's cell (deduplicated), returns the count. */
static int grid_neighbours(const sph_params *p, const grid_t *g, const double *ri,
                           int64_t *cells) {
    int d = p->dim;
    int cc[3] = {0, 0, 0};
    for (int a = 0; a < d; ++a) {
        double L = p->box[a];
        double x = ri[a] - L * floor(ri[a] / L);
        int ci = (int)(x / g->edge[a]);
        if (ci < 0) ci = 0;
        if (ci >= g->nc[a]) ci = g->nc[a] - 1;
        cc[a] = ci;
    }
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        if (a < d && g->nc[a] >= 3) {
            lo[a] = -1;
            hi[a] = 1;
        } else {
            lo[a] = 0;
            hi[a] = 0;
        }
    }
    int k = 0;
    for (int oz = lo[2]; oz <= hi[2]; ++oz)
        for (int oy = lo[1]; oy <= hi[1]; ++oy)
            for (int ox = lo[0]; ox <= hi[0]; ++ox) {
                int o[3] = {ox, oy, oz};
                int64_t c = 0;
                for (int a = d - 1; a >= 0; --a) {
                    int x = cc[a] + o[a];
                    if (x < 0) x += g->nc[a];
                    if (x >= g->nc[a]) x -= g->nc[a];
                    c = c * g->nc[a] + x;
                }
                cells[k++] = c;
            }
    return k;
}

/* Calls fn(i, j, dr, rsq) for every j != i in the pair set, j ascending
 * within each cell. */
#define FOR_NEIGHBOURS(P, G, N, R, I, ...)                                        \
    do {                                                                           \
        int64_t _cells[27];                                                        \
        int _nc = grid_neighbours((P), (G), &(R)[(I) * (P)->dim], _cells);         \
        double _thr = pair_threshold(P);                                           \
        for (int _k = 0; _k < _nc; ++_k) {                                         \
            int64_t _c = _cells[_k];                                               \
            for (int64_t _s = (G)->start[_c]; _s < (G)->start[_c + 1]; ++_s) {     \
                int64_t j = (G)->idx[_s];                                          \
                if (j == (I)) continue;                                            \
                double dr[3] = {0, 0, 0};                                          \
                double rsq = pair_rsq((P), &(R)[(I) * (P)->dim], &(R)[j * (P)->dim], dr); \
                if (!(rsq < _thr)) continue;                                       \
                if (g_geom32) geometry32((P)->dim, dr, &rsq);                      \
                __VA_ARGS__                                                        \
            }                                                                      \
        }                                                                          \
    } while (0)

/* ---- pair set ----------------------------------------------------------- */

/* Brute force i<j row-major, the order of VerletList.build. */
int orc_pairs_brute(const sph_params *p, int64_t n, const double *r, int64_t cap,
                    int64_t *iap, double *rsq_out, int64_t *nip) {
    double thr = pair_threshold(p);
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = i + 1; j < n; ++j) {
            double dr[3];
            double rsq = pair_rsq(p, &r[i * p->dim], &r[j * p->dim], dr);
            if (rsq < thr) {
                if (k < cap) {
                    if (iap) {
                        iap[2 * k] = i;
                        iap[2 * k + 1] = j;
                    }
                    if (rsq_out) rsq_out[k] = rsq;
                }
                ++k;
            }
        }
    *nip = k;
    return k > cap ? SPH_ECAPACITY : SPH_OK;
}

static int cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/* Cell-list pair set, same pairs as orc_pairs_brute, ordered by (i, j). */
int orc_pairs(const sph_params *p, int64_t n, const double *r, int64_t cap, int64_t *iap,
              double *rsq_out, int64_t *nip) {
    grid_t g;
    int st = grid_build(p, n, r, &g);
    if (st) return st;
    int64_t *cnt = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
#pragma omp parallel for schedule(dynamic, 256) num_threads(orc_get_threads())
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        FOR_NEIGHBOURS(p, &g, n, r, i, { if (j > i) ++c; });
        cnt[i + 1] = c;
    }
    for (int64_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    *nip = cnt[n];
    if (cnt[n] > cap) {
        free(cnt);
        grid_free(&g);
        return SPH_ECAPACITY;
    }
    if (iap || rsq_out) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(orc_get_threads())
        for (int64_t i = 0; i < n; ++i) {
            int64_t base = cnt[i], m = 0;
            int64_t *js = (int64_t *)malloc(sizeof(int64_t) * (size_t)(cnt[i + 1] - base + 1));
            FOR_NEIGHBOURS(p, &g, n, r, i, { if (j > i) js[m++] = j; });
            qsort(js, (size_t)m, sizeof(int64_t), cmp_i64);
            for (int64_t t = 0; t < m; ++t) {
                if (iap) {
                    iap[2 * (base + t)] = i;
                    iap[2 * (base + t) + 1] = js[t];
                }
                if (rsq_out) {
                    double dr[3];
                    rsq_out[base + t] = pair_rsq(p, &r[i * p->dim], &r[js[t] * p->dim], dr);
                }
            }
            free(js);
        }
    }
    free(cnt);
    grid_free(&g);
    return SPH_OK;
}

/* ---- hard collisions ---------------------------------------------------- */

/* One pair of the sequential loop (forces.py:87-156 and 158-243). */
static void collide_pair(int dim, int mode, double *r, double *v, const double *m, int64_t i,
                         int64_t j, double *dr, double *rij, double cutoff) {
    double *vi = &v[i * dim], *vj = &v[j * dim];
    double drsq = dr[0] * dr[0];
    double vidotr = vi[0] * dr[0], vjdotr = vj[0] * dr[0];
    for (int a = 1; a < dim; ++a) {
        drsq = drsq + dr[a] * dr[a];
        vidotr = vidotr + vi[a] * dr[a];
        vjdotr = vjdotr + vj[a] * dr[a];
    }
    if (vidotr < 0 && vjdotr > 0) return;
    double vti[3], vni[3], vtj[3], vnj[3];
    for (int a = 0; a < dim; ++a) {
        vti[a] = (vidotr / drsq) * dr[a];
        vni[a] = vi[a] - vti[a];
        vtj[a] = (vjdotr / drsq) * dr[a];
        vnj[a] = vj[a] - vtj[a];
    }
    for (int a = 0; a < dim; ++a) {
        double tmp = vti[a];
        vti[a] = vtj[a] * (m[j] / m[i]);
        vtj[a] = tmp * (m[i] / m[j]);
    }
    for (int a = 0; a < dim; ++a) {
        vi[a] = vti[a] + vni[a];
        vj[a] = vtj[a] + vnj[a];
    }
    if (mode == SPH_COLLIDE_PUSHBACK && drsq < cutoff * cutoff) {
        double ro = (cutoff + 0.01 - *rij) / 2.0, nsq = 0.0;
        for (int a = 0; a < dim; ++a) {
            double dro = (dr[a] / *rij) * ro;
            r[i * dim + a] -= dro;
            r[j * dim + a] += dro;
        }
        for (int a = 0; a < dim; ++a) {
            dr[a] = r[j * dim + a] - r[i * dim + a];
            nsq = a == 0 ? dr[a] * dr[a] : nsq + dr[a] * dr[a];
        }
        *rij = sqrt(nsq);
    }
}

/* Force.apply of a collision force over a pair list (forces.py:38-42). */
int orc_collide_pairs(int32_t dim, int32_t mode, int64_t n, double *r, double *v,
                      const double *m, int64_t nip, const int64_t *iap, double *drij,
                      double *rij, double cutoff) {
    double c2 = cutoff * cutoff;
    for (int64_t k = 0; k < nip; ++k) {
        int64_t i = iap[2 * k], j = iap[2 * k + 1];
        if (i < 0 || j < 0 || i >= n || j >= n || i == j) return SPH_EINVAL;
        if (rij[k] * rij[k] <= c2)
            collide_pair(dim, mode, r, v, m, i, j, &drij[k * dim], &rij[k], cutoff);
    }
    return SPH_OK;
}

/* Collisions of one evaluation: the pair set at r in (i, j) order. */
static int collide_state(const sph_params *p, int64_t n, double *r, double *v,
                         const double *m) {
    int64_t nip = 0;
    int st = orc_pairs(p, n, r, 0, NULL, NULL, &nip);
    if (st != SPH_OK && st != SPH_ECAPACITY) return st;
    int64_t *iap = malloc(sizeof(int64_t) * 2 * (size_t)(nip + 1));
    double *rsq = malloc(sizeof(double) * (size_t)(nip + 1));
    st = orc_pairs(p, n, r, nip, iap, rsq, &nip);
    double c2 = p->collision_cutoff * p->collision_cutoff;
    for (int64_t k = 0; st == SPH_OK && k < nip; ++k) {
        double rij = sqrt(rsq[k]);
        if (!(rij * rij <= c2)) continue;
        double dr[3];
        pair_rsq(p, &r[iap[2 * k] * p->dim], &r[iap[2 * k + 1] * p->dim], dr);
        collide_pair(p->dim, SPH_COLLIDE_EXCHANGE, r, v, m, iap[2 * k], iap[2 * k + 1], dr,
                     &rij, p->collision_cutoff);
    }
    free(iap);
    free(rsq);
    return st;
}

/* ---- one derivative evaluation (gather form, OpenMP over particles) ----- */

typedef struct {
    double *rho, *rho_lr, *t, *pres, *pco, *vdot, *udot, *jq;
} orc_out;

static int derivatives(const sph_params *p, int64_t n, const double *r, const double *v,
                       const double *m, const double *u, orc_out *o, int64_t *nip) {
    int d = p->dim;
    int kt = p->kernel;
    double hs = p->h_short, hl = p->h_long;
    grid_t g;
    int st = grid_build(p, n, r, &g);
    if (st) return st;
    double ws0, wl0, dummy;
    kern(kt, d, 0.0, hs, &ws0, &dummy);
    kern(kt, d, 0.0, hl, &wl0, &dummy);
    int64_t pairs2 = 0;
    /* pass 1: densities and the equation of state */
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : pairs2) num_threads(orc_get_threads())
    for (int64_t i = 0; i < n; ++i) {
        double rs = ws0, rl = wl0;
        int64_t c = 0;
        FOR_NEIGHBOURS(p, &g, n, r, i, {
            double rr = sqrt(rsq), w, gg;
            kern(kt, d, rr, hs, &w, &gg);
            rs += w * m[j];
            kern(kt, d, rr, hl, &w, &gg);
            rl += w * m[j];
            ++c;
        });
        pairs2 += c;
        o->rho[i] = rs;
        o->rho_lr[i] = rl;
        double T = (u[i] + p->adash * rs) / p->kbdash;
        if (T < 0.0) T = 0.0;
        o->t[i] = T;
        o->pres[i] = (rs * p->kbdash * T) / (1 - rs * p->bdash);
        o->pco[i] = -p->adash * rl * rl;
    }
    /* pass 2: heat flux vector */
    if (p->heat_flux) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(orc_get_threads())
        for (int64_t i = 0; i < n; ++i) {
            double q[3] = {0, 0, 0};
            FOR_NEIGHBOURS(p, &g, n, r, i, {
                double rr = sqrt(rsq), w, gg;
                kern(kt, d, rr, hs, &w, &gg);
                double f = p->thermalk * (m[j] / o->rho[j]) * (o->t[j] - o->t[i]) * gg;
                for (int a = 0; a < d; ++a) q[a] += f * dr[a];
            });
            for (int a = 0; a < d; ++a) o->jq[i * d + a] = q[a];
        }
    } else if (o->jq) {
        memset(o->jq, 0, sizeof(double) * (size_t)(n * d));
    }
    /* pass 3: forces and energy rates */
#pragma omp parallel for schedule(dynamic, 256) num_threads(orc_get_threads())
    for (int64_t i = 0; i < n; ++i) {
        double acc[3] = {0, 0, 0}, ud = 0.0;
        double fsi = o->pres[i] / (o->rho[i] * o->rho[i]);
        double fli = o->pco[i] / (o->rho_lr[i] * o->rho_lr[i]);
        FOR_NEIGHBOURS(p, &g, n, r, i, {
            double rr = sqrt(rsq), w, gs, gl;
            kern(kt, d, rr, hs, &w, &gs);
            kern(kt, d, rr, hl, &w, &gl);
            double dv[3] = {0, 0, 0}, dvdr = 0.0;
            for (int a = 0; a < d; ++a) {
                dv[a] = v[j * d + a] - v[i * d + a];
                dvdr += dv[a] * dr[a];
            }
            double ps = fsi + o->pres[j] / (o->rho[j] * o->rho[j]);
            if (p->viscosity && dvdr < 0.0) {
                double mu = hs * dvdr / (rsq + p->visc_eps * hs * hs);
                double rbar = 0.5 * (o->rho[i] + o->rho[j]);
                ps += (-p->visc_alpha * p->sound_speed * mu + p->visc_beta * mu * mu) / rbar;
            }
            double pl = fli + o->pco[j] / (o->rho_lr[j] * o->rho_lr[j]);
            double du_s = 0.0, du_l = 0.0;
            for (int a = 0; a < d; ++a) {
                double as = ps * (gs * dr[a]);
                double al = pl * (gl * dr[a]);
                acc[a] += as;
                acc[a] += al;
                du_s += as * dv[a];
                du_l += al * dv[a];
            }
            ud += 0.5 * du_s * m[j];
            ud += 0.5 * du_l * m[j];
            if (p->heat_flux) {
                double dq = 0.0;
                for (int a = 0; a < d; ++a) {
                    double qa = o->jq[i * d + a] / (o->rho[i] * o->rho[i]) +
                                o->jq[j * d + a] / (o->rho[j] * o->rho[j]);
                    dq += qa * (gs * dr[a]);
                }
                ud -= dq * m[j];
            }
        });
        for (int a = 0; a < d; ++a) o->vdot[i * d + a] = acc[a];
        o->udot[i] = ud;
    }
    grid_free(&g);
    if (nip) *nip = pairs2 / 2;
    return SPH_OK;
}

int orc_derivatives(const sph_params *p, int64_t n, const double *r, const double *v,
                    const double *m, const double *u, double *rho, double *rho_lr, double *t,
                    double *pres, double *pco, double *vdot, double *udot, double *jq,
                    int64_t *nip) {
    if (p->dim < 2 || p->dim > 3) return SPH_EINVAL;
    int d = p->dim;
    double *tmp_jq = NULL;
    if (!jq) {
        tmp_jq = (double *)calloc((size_t)(n * d + 1), sizeof(double));
        jq = tmp_jq;
    }
    orc_out o = {rho, rho_lr, t, pres, pco, vdot, udot, jq};
    int st = derivatives(p, n, r, v, m, u, &o, nip);
    free(tmp_jq);
    return st;
}

/* ---- integrator + box + thermostat --------------------------------------- */

static void teleport(const sph_params *p, int64_t n, double *r) {
    int d = p->dim;
    for (int64_t i = 0; i < n; ++i)
        for (int a = 0; a < d; ++a) {
            double L = p->box[a];
            if (r[i * d + a] > L) r[i * d + a] = 0;
            if (r[i * d + a] < 0) r[i * d + a] = L;
        }
}

static double thermostat_target(const sph_params *p, int64_t step_done) {
    if (p->thermostat_ramp_steps <= 0) return p->thermostat_temp;
    double f = (double)step_done / (double)p->thermostat_ramp_steps;
    if (f > 1.0) f = 1.0;
    return p->thermostat_temp + (p->thermostat_temp_end - p->thermostat_temp) * f;
}

/* Advances nsteps.  step0 is the number of steps already taken (thermostat
 * ramp).  On return rho/pres/pco hold the last step's first evaluation,
 * t/rho_lr/vdot/udot/jq its last evaluation (reference semantics). */
int orc_advance(const sph_params *p, int64_t n, double *r, double *v, const double *m,
                double *u, int32_t nsteps, int64_t step0, double *rho, double *rho_lr,
                double *t, double *pres, double *pco, double *vdot, double *udot, double *jq) {
    int d = p->dim;
    size_t nd = (size_t)(n * d), n1 = (size_t)n;
    double *r0 = malloc(sizeof(double) * nd), *v0 = malloc(sizeof(double) * nd);
    double *u0 = malloc(sizeof(double) * n1);
    double *cr = malloc(sizeof(double) * nd * 4), *cv = malloc(sizeof(double) * nd * 4);
    double *cu = malloc(sizeof(double) * n1 * 4);
    double *rho0 = malloc(sizeof(double) * n1), *p0 = malloc(sizeof(double) * n1);
    double *pco0 = malloc(sizeof(double) * n1);
    double *ojq = jq ? jq : calloc(nd + 1, sizeof(double));
    int st = SPH_OK;
    int nstage = p->integrator == SPH_EULER ? 1 : (p->integrator == SPH_RK4 ? 4 : 2);
    const int coll = p->collision == SPH_COLLIDE_EXCHANGE;
    for (int32_t s = 0; s < nsteps && st == SPH_OK; ++s) {
        if (coll) {
            /* update()'s extra first evaluation: only its collisions remain */
            st = collide_state(p, n, r, v, m);
            if (st) break;
        }
        memcpy(r0, r, sizeof(double) * nd);
        memcpy(v0, v, sizeof(double) * nd);
        memcpy(u0, u, sizeof(double) * n1);
        for (int k = 0; k < nstage; ++k) {
            orc_out o = {rho, rho_lr, t, pres, pco, vdot, udot, ojq};
            st = derivatives(p, n, r, v, m, u, &o, NULL);
            if (st) break;
            if (coll) {
                st = collide_state(p, n, r, v, m);
                if (st) break;
                if (k == 0) memcpy(v0, v, sizeof(double) * nd);  /* x_start */
            }
            if (k == 0) {
                memcpy(rho0, rho, sizeof(double) * n1);
                memcpy(p0, pres, sizeof(double) * n1);
                memcpy(pco0, pco, sizeof(double) * n1);
            }
            /* c_k = xdot * dt */
            for (size_t i = 0; i < nd; ++i) {
                cr[k * nd + i] = v[i] * p->dt;
                cv[k * nd + i] = vdot[i] * p->dt;
            }
            for (size_t i = 0; i < n1; ++i) cu[k * n1 + i] = udot[i] * p->dt;
            if (p->integrator == SPH_EULER) {
                for (size_t i = 0; i < nd; ++i) {
                    r[i] = r0[i] + cr[i];
                    v[i] = v0[i] + cv[i];
                }
                for (size_t i = 0; i < n1; ++i) u[i] = u0[i] + cu[i];
            } else if (p->integrator == SPH_IEULER) {
                if (k == 0) {
                    for (size_t i = 0; i < nd; ++i) {
                        r[i] = r0[i] + cr[i];
                        v[i] = v0[i] + cv[i];
                    }
                    for (size_t i = 0; i < n1; ++i) u[i] = u0[i] + cu[i];
                } else {
                    for (size_t i = 0; i < nd; ++i) {
                        r[i] = r0[i] + (cr[i] + cr[nd + i]) / 2;
                        v[i] = v0[i] + (cv[i] + cv[nd + i]) / 2;
                    }
                    for (size_t i = 0; i < n1; ++i) u[i] = u0[i] + (cu[i] + cu[n1 + i]) / 2;
                }
            } else { /* rk4, integrator.py:62-103 */
                if (k < 2) {
                    for (size_t i = 0; i < nd; ++i) {
                        r[i] = r0[i] + cr[k * nd + i] / 2.0;
                        v[i] = v0[i] + cv[k * nd + i] / 2.0;
                    }
                    for (size_t i = 0; i < n1; ++i) u[i] = u0[i] + cu[k * n1 + i] / 2.0;
                } else if (k == 2) {
                    for (size_t i = 0; i < nd; ++i) {
                        r[i] = r0[i] + cr[2 * nd + i];
                        v[i] = v0[i] + cv[2 * nd + i];
                    }
                    for (size_t i = 0; i < n1; ++i) u[i] = u0[i] + cu[2 * n1 + i];
                } else {
                    for (size_t i = 0; i < nd; ++i) {
                        r[i] = r0[i] + (1.0 / 6.0) * (cr[i] + 2. * cr[nd + i] + 2. * cr[2 * nd + i] + cr[3 * nd + i]);
                        v[i] = v0[i] + (1.0 / 6.0) * (cv[i] + 2. * cv[nd + i] + 2. * cv[2 * nd + i] + cv[3 * nd + i]);
                    }
                    for (size_t i = 0; i < n1; ++i)
                        u[i] = u0[i] + (1.0 / 6.0) * (cu[i] + 2. * cu[n1 + i] + 2. * cu[2 * n1 + i] + cu[3 * n1 + i]);
                }
            }
        }
        if (st) break;
        teleport(p, n, r);
        memcpy(rho, rho0, sizeof(double) * n1);
        memcpy(pres, p0, sizeof(double) * n1);
        memcpy(pco, pco0, sizeof(double) * n1);
        if (p->thermostat) {
            double tav = 0.0;
            for (size_t i = 0; i < n1; ++i) tav += t[i];
            tav /= (double)n1;
            double scale = thermostat_target(p, step0 + s + 1) / tav;
            for (size_t i = 0; i < n1; ++i) {
                t[i] = t[i] * scale;
                u[i] = t[i] * p->kbdash - p->adash * rho[i];
            }
        }
    }
    free(r0); free(v0); free(u0); free(cr); free(cv); free(cu);
    free(rho0); free(p0); free(pco0);
    if (!jq) free(ojq);
    return st;
}

/* Kernel value and gradient factor for tests of the kernel tables. */
void orc_kernel(int type, int dim, double r, double h, double *w, double *g) {
    kern(type, dim, r, h, w, g);
}
