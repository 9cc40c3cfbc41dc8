/*
 * mdg_oracle.c -- CPU oracle for the force-and-step path.  TEST INFRASTRUCTURE:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load
 * this library, and only to check (or time on the host) what the CUDA path
 * computes.  The shipped package never calls it.
 *
 * Everything is FP64 unless a function says otherwise.  Each function names
 * the reference code it restates (paths relative to the mdpy v0.2.1 tree):
 *
 *   orc_ref_cell_index      mdpy/core/cell_list.py:74-116   (CellList geometry + kernel)
 *   orc_ref_pairs           mdpy/constraint/charmm_nonbonded_constraint.py:75-90
 *                           (27-cell template walk, exclusions, r <= rc)
 *   orc_ref_lj              charmm_nonbonded_constraint.py:64-108 (LJ, 1-4 params, hard cutoff)
 *   orc_ref_coulomb         mdpy/constraint/electrostatic_constraint.py:52-79 (all pairs, min image)
 *   orc_nonbonded           LJ (+ optional CHARMM switch) and Ewald real-space erfc;
 *                           no reference counterpart (mdpy has no Ewald), restated from
 *                           the Ewald decomposition
 *   orc_ewald_recip         direct reciprocal-space Ewald k-sum (no reference counterpart)
 *   orc_ewald_exclusions    -qq erf(beta r)/r for excluded pairs (no reference counterpart)
 *   orc_pme_spread/gather   order-p cardinal B-spline PME (Essmann et al. 1995)
 *   orc_bonds / orc_angles  mdpy/constraint/charmm_bond_constraint.py:52-73,
 *                           charmm_angle_constraint.py:138-179
 *   orc_dihedrals           V = k(1+cos(n phi - delta)) with the exact gradient; the
 *                           reference's force (charmm_dihedral_constraint.py:81) is not
 *                           -dV/dphi and is not followed
 *   orc_impropers           V = k(psi-psi0)^2, exact gradient
 *                           (charmm_improper_constraint.py:57-93)
 *   orc_philox4x32          Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)
 *   orc_langevin_noise      Box-Muller normals from Philox, float32 (same recipe as
 *                           the device integrator)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_API __attribute__((visibility("default")))

static inline double wrap1(double d, double L) { return d - L * nearbyint(d / L); }

int ORC_API orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void ORC_API orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* reference cell list (float32, exactly the reference's arithmetic)        */
/* ------------------------------------------------------------------------ */
/*
 * CellList._update_attributes (cell_list.py:74-81): n_d = max(3, floor((L_d +
 * skin)/rc)), cell edge (L_d + skin)/n_d stored as float32, cell_inv its
 * inverse.  CellList.update (:83-90) shifts positions by their per-axis
 * minimum and takes floor(x * cell_inv) (:99).
 */
int ORC_API orc_ref_cell_index(const float *pos, int n, const float *pbc_diag, float cutoff,
                               float skin, int *num_cell_vec, int *cell_index) {
    float mins[3] = {INFINITY, INFINITY, INFINITY};
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d)
            if (pos[3 * i + d] < mins[d]) mins[d] = pos[3 * i + d];
    for (int d = 0; d < 3; ++d) {
        int nc = (int)floor(((double)pbc_diag[d] + (double)skin) / (double)cutoff);
        if (nc < 3) nc = 3;
        num_cell_vec[d] = nc;
    }
    for (int d = 0; d < 3; ++d) {
        float edge = (float)(((double)pbc_diag[d] + (double)skin) / (double)num_cell_vec[d]);
        float inv = 1.0f / edge;
        for (int i = 0; i < n; ++i) {
            float p = pos[3 * i + d] - mins[d];
            cell_index[3 * i + d] = (int)floorf(p * inv);
        }
    }
    return 0;
}

static inline int is_listed(const int *row, int width, int j) {
    for (int k = 0; k < width; ++k)
        if (row[k] == j) return 1;
    return 0;
}

/*
 * The reference's pair test in its own float32 arithmetic: d = x_j - x_i,
 * scaled by the float32 inverse box, minus its rounded value, scaled back
 * (unwrap_vec, mdpy/utils/pbc.py:38-43), r = sqrt of the left-to-right sum
 * of squares (np.linalg.norm, charmm_nonbonded_constraint.py:85-90), r <= rc.
 * Every operation rounds once (the library is built with -ffp-contract=off,
 * so no multiply-add is fused on any host).
 */
static inline int ref_within32(const float *pos, int i, int j, const float *pbc_diag,
                               float cutoff) {
    float d[3];
    for (int k = 0; k < 3; ++k) {
        float L = pbc_diag[k];
        float s = (pos[3 * j + k] - pos[3 * i + k]) * (1.0f / L);
        s = s - rintf(s);
        d[k] = s * L;
    }
    float r = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    return r <= cutoff;
}

/* all unordered pairs i<j (not excluded) that pass ref_within32: the set the
 * reference's kernel would visit if its cell walk missed no periodic
 * neighbour; all pairs, O(n^2) */
long ORC_API orc_pairs_bruteforce_ref32(const float *pos, int n, const float *pbc_diag,
                                        float cutoff, const int *excl, int excl_width,
                                        int *pairs_out, long cap) {
    long np = 0;
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            if (excl_width > 0 && is_listed(excl + (long)i * excl_width, excl_width, j)) continue;
            if (!ref_within32(pos, i, j, pbc_diag, cutoff)) continue;
            if (np < cap) {
                pairs_out[2 * np] = i;
                pairs_out[2 * np + 1] = j;
            }
            ++np;
        }
    return np;
}

/*
 * Pairs the reference's nonbonded kernel visits with r <= rc
 * (charmm_nonbonded_constraint.py:75-90): j lies in one of the 27 cells
 * (c_i + t) mod n (the kernel subtracts n for indices >= n and relies on
 * negative indexing for -1), j != i, j not in bonded_particles[i], and the
 * minimum-image distance (float32, unwrap_vec at mdpy/utils/pbc.py:38-43)
 * is <= rc.  Returns unordered pairs i<j; capacity-checked.
 */
long ORC_API orc_ref_pairs(const float *pos, int n, const float *pbc_diag, float cutoff,
                           const int *cell_index, const int *num_cell_vec,
                           const int *excl, int excl_width, int *pairs_out, long cap) {
    const int nx = num_cell_vec[0], ny = num_cell_vec[1], nz = num_cell_vec[2];
    const long ncell = (long)nx * ny * nz;
    int *count = calloc(ncell, sizeof(int));
    for (int i = 0; i < n; ++i) {
        const int *c = cell_index + 3 * i;
        count[((long)c[0] * ny + c[1]) * nz + c[2]]++;
    }
    long *start = malloc((ncell + 1) * sizeof(long));
    start[0] = 0;
    for (long c = 0; c < ncell; ++c) start[c + 1] = start[c] + count[c];
    int *members = malloc((size_t)n * sizeof(int));
    memset(count, 0, ncell * sizeof(int));
    for (int i = 0; i < n; ++i) {
        const int *c = cell_index + 3 * i;
        long cc = ((long)c[0] * ny + c[1]) * nz + c[2];
        members[start[cc] + count[cc]++] = i;
    }
    long np = 0;
    for (int i = 0; i < n; ++i) {
        const int *ci = cell_index + 3 * i;
        /* n >= 3 per axis, so t in {-1,0,1} gives 3 distinct cells per axis */
        for (int tx = -1; tx <= 1; ++tx)
            for (int ty = -1; ty <= 1; ++ty)
                for (int tz = -1; tz <= 1; ++tz) {
                    int cx = (ci[0] + tx + nx) % nx, cy = (ci[1] + ty + ny) % ny,
                        cz = (ci[2] + tz + nz) % nz;
                    long cc = ((long)cx * ny + cy) * nz + cz;
                    for (long m = start[cc]; m < start[cc + 1]; ++m) {
                        int j = members[m];
                        if (j <= i) continue;
                        if (excl_width > 0 && is_listed(excl + (long)i * excl_width, excl_width, j))
                            continue;
                        if (ref_within32(pos, i, j, pbc_diag, cutoff)) {
                            if (np < cap) {
                                pairs_out[2 * np] = i;
                                pairs_out[2 * np + 1] = j;
                            }
                            ++np;
                        }
                    }
                }
    }
    free(count);
    free(start);
    free(members);
    return np;
}

/* ------------------------------------------------------------------------ */
/* generic FP64 neighbour search (cells >= rc, or all pairs)                */
/* ------------------------------------------------------------------------ */
typedef struct {
    int nc[3];
    int *start, *members;
    int brute;
} cellgrid;

static void grid_build(cellgrid *g, const double *pos, int n, const double *box, double rc) {
    g->brute = 0;
    for (int d = 0; d < 3; ++d) {
        g->nc[d] = (int)floor(box[d] / rc);
        if (g->nc[d] < 3) g->brute = 1;
    }
    if (g->brute) {
        g->nc[0] = g->nc[1] = g->nc[2] = 1;
    }
    long ncell = (long)g->nc[0] * g->nc[1] * g->nc[2];
    g->start = calloc(ncell + 1, sizeof(int));
    g->members = malloc((size_t)n * sizeof(int));
    int *cell = malloc((size_t)n * sizeof(int));
    for (int i = 0; i < n; ++i) {
        int c[3];
        for (int d = 0; d < 3; ++d) {
            double x = pos[3 * i + d] - box[d] * floor(pos[3 * i + d] / box[d]);
            int k = (int)(x / box[d] * g->nc[d]);
            if (k >= g->nc[d]) k = g->nc[d] - 1;
            if (k < 0) k = 0;
            c[d] = k;
        }
        cell[i] = (c[0] * g->nc[1] + c[1]) * g->nc[2] + c[2];
        g->start[cell[i] + 1]++;
    }
    for (long c = 0; c < ncell; ++c) g->start[c + 1] += g->start[c];
    int *fill = calloc(ncell, sizeof(int));
    for (int i = 0; i < n; ++i) g->members[g->start[cell[i]] + fill[cell[i]]++] = i;
    free(fill);
    free(cell);
}

static void grid_free(cellgrid *g) {
    free(g->start);
    free(g->members);
}

static inline int grid_cell_of(const cellgrid *g, const double *p, const double *box, int *c) {
    for (int d = 0; d < 3; ++d) {
        double x = p[d] - box[d] * floor(p[d] / box[d]);
        int k = (int)(x / box[d] * g->nc[d]);
        if (k >= g->nc[d]) k = g->nc[d] - 1;
        if (k < 0) k = 0;
        c[d] = k;
    }
    return 0;
}

/* Iterate the 27 neighbour cells (or the single cell) of atom i. */
#define FOR_NEIGHBOURS(g, box, pos, i, j, ...)                                          \
    do {                                                                                 \
        int _c[3];                                                                       \
        grid_cell_of(&(g), (pos) + 3 * (i), (box), _c);                                  \
        int _r = (g).brute ? 0 : 1;                                                      \
        for (int _tx = -_r; _tx <= _r; ++_tx)                                            \
            for (int _ty = -_r; _ty <= _r; ++_ty)                                        \
                for (int _tz = -_r; _tz <= _r; ++_tz) {                                  \
                    int _cx = (_c[0] + _tx + (g).nc[0]) % (g).nc[0];                     \
                    int _cy = (_c[1] + _ty + (g).nc[1]) % (g).nc[1];                     \
                    int _cz = (_c[2] + _tz + (g).nc[2]) % (g).nc[2];                     \
                    long _cc = ((long)_cx * (g).nc[1] + _cy) * (g).nc[2] + _cz;          \
                    for (int _m = (g).start[_cc]; _m < (g).start[_cc + 1]; ++_m) {       \
                        int j = (g).members[_m];                                         \
                        __VA_ARGS__                                                      \
                    }                                                                    \
                }                                                                        \
    } while (0)

/* all unordered pairs i<j within rc under the minimum image (FP64) */
long ORC_API orc_pairs_bruteforce(const double *pos, int n, const double *box, double rc,
                                  int *pairs_out, long cap) {
    cellgrid g;
    grid_build(&g, pos, n, box, rc);
    long np = 0;
    double rc2 = rc * rc;
    for (int i = 0; i < n; ++i) {
        FOR_NEIGHBOURS(g, box, pos, i, j, {
            if (j > i) {
                double r2 = 0;
                for (int d = 0; d < 3; ++d) {
                    double dd = wrap1(pos[3 * j + d] - pos[3 * i + d], box[d]);
                    r2 += dd * dd;
                }
                if (r2 <= rc2) {
                    if (np < cap) {
                        pairs_out[2 * np] = i;
                        pairs_out[2 * np + 1] = j;
                    }
                    ++np;
                }
            }
        });
    }
    grid_free(&g);
    return np;
}

/* ------------------------------------------------------------------------ */
/* nonbonded: LJ (+switch) and Coulomb                                       */
/* ------------------------------------------------------------------------ */
/*
 * params: per atom (eps, sigma, eps14, sigma14); combination eps = sqrt(eps_i
 * eps_j), sigma = (sigma_i + sigma_j)/2 (charmm_nonbonded_constraint.py:98-101).
 * Pairs listed in `excl` (1-2, 1-3) are skipped; pairs listed in `scal` (1-4)
 * use the 14 parameters.  V_LJ = 4 eps (s^12 - s^6) with hard cutoff at rc
 * (reference, :90,107), optionally multiplied by the CHARMM switch
 * S(r) = (rc^2-r^2)^2 (rc^2+2r^2-3rs^2)/(rc^2-rs^2)^3 on rs < r <= rc.
 *
 * coul_mode 0: no Coulomb; 1: Ewald real space k qq erfc(beta r)/r inside rc;
 * 2: bare Coulomb k qq / r over ALL pairs (minimum image, no cutoff) as
 * electrostatic_constraint.py:52-79.
 *
 * Full-neighbour loop, forces on i only, each pair energy counted half per
 * visit: thread-safe and order-deterministic under a static schedule.
 * energies[0] = LJ, energies[1] = Coulomb.
 */
/*
 * orc_nonbonded_rows: the same loop for the atoms rows[0..nrows) only (forces
 * (nrows, 3) on those atoms; energies count only the pairs visited from
 * them).  rows == NULL means every atom in order.
 */
void ORC_API orc_nonbonded_rows(const double *pos, int n, const double *box,
                                const double *params, const double *q, const int *excl,
                                int excl_width, const int *scal, int scal_width, double rc,
                                double rs, int use_switch, int lj_on, int coul_mode, double beta,
                                double kcoul, const int *rows, int nrows, double *forces,
                                double *energies);

void ORC_API orc_nonbonded(const double *pos, int n, const double *box, const double *params,
                           const double *q, const int *excl, int excl_width, const int *scal,
                           int scal_width, double rc, double rs, int use_switch, int lj_on,
                           int coul_mode, double beta, double kcoul, double *forces,
                           double *energies) {
    orc_nonbonded_rows(pos, n, box, params, q, excl, excl_width, scal, scal_width, rc, rs,
                       use_switch, lj_on, coul_mode, beta, kcoul, NULL, n, forces, energies);
}

void ORC_API orc_nonbonded_rows(const double *pos, int n, const double *box,
                                const double *params, const double *q, const int *excl,
                                int excl_width, const int *scal, int scal_width, double rc,
                                double rs, int use_switch, int lj_on, int coul_mode, double beta,
                                double kcoul, const int *rows, int nrows, double *forces,
                                double *energies) {
    cellgrid g;
    double search = (coul_mode == 2) ? 1e300 : rc;
    if (coul_mode == 2) {
        g.brute = 1;
        g.nc[0] = g.nc[1] = g.nc[2] = 1;
        g.start = calloc(2, sizeof(int));
        g.start[1] = n;
        g.members = malloc((size_t)n * sizeof(int));
        for (int i = 0; i < n; ++i) g.members[i] = i;
    } else {
        grid_build(&g, pos, n, box, search);
    }
    const double rc2 = rc * rc, rs2 = rs * rs;
    const double two_over_sqrtpi = 1.1283791670955126;
    double e_lj = 0, e_c = 0;
#pragma omp parallel for schedule(static) reduction(+ : e_lj, e_c)
    for (int r = 0; r < nrows; ++r) {
        const int i = rows ? rows[r] : r;
        double fi[3] = {0, 0, 0};
        const int *xrow = excl_width > 0 ? excl + (long)i * excl_width : NULL;
        const int *srow = scal_width > 0 ? scal + (long)i * scal_width : NULL;
        FOR_NEIGHBOURS(g, box, pos, i, j, {
            if (j != i && !(xrow && is_listed(xrow, excl_width, j))) {
                double d[3], r2 = 0;
                for (int k = 0; k < 3; ++k) {
                    d[k] = wrap1(pos[3 * j + k] - pos[3 * i + k], box[k]);
                    r2 += d[k] * d[k];
                }
                double fr = 0; /* -dV/dr / r : force on j is +fr*d, on i is -fr*d */
                if (lj_on && r2 <= rc2) {
                    int s14 = srow && is_listed(srow, scal_width, j);
                    double ei = params[4 * i + (s14 ? 2 : 0)], si = params[4 * i + (s14 ? 3 : 1)];
                    double ej = params[4 * j + (s14 ? 2 : 0)], sj = params[4 * j + (s14 ? 3 : 1)];
                    double eps = sqrt(ei * ej), sig = 0.5 * (si + sj);
                    double s2 = sig * sig / r2, s6 = s2 * s2 * s2;
                    double v = 4 * eps * (s6 * s6 - s6);
                    double f = 24 * eps * (2 * s6 * s6 - s6) / r2;
                    if (use_switch && r2 > rs2) {
                        double den = (rc2 - rs2) * (rc2 - rs2) * (rc2 - rs2);
                        double sw = (rc2 - r2) * (rc2 - r2) * (rc2 + 2 * r2 - 3 * rs2) / den;
                        double dsw = 12 * (rc2 - r2) * (rs2 - r2) / den; /* dS/dr / r */
                        f = f * sw - v * dsw;
                        v *= sw;
                    }
                    e_lj += 0.5 * v;
                    fr += f;
                }
                if (coul_mode == 1 && r2 <= rc2) {
                    double r = sqrt(r2), qq = kcoul * q[i] * q[j];
                    double ec = erfc(beta * r);
                    e_c += 0.5 * qq * ec / r;
                    fr += qq * (ec / r + beta * two_over_sqrtpi * exp(-beta * beta * r2)) / r2;
                } else if (coul_mode == 2) {
                    double r = sqrt(r2), qq = kcoul * q[i] * q[j];
                    e_c += 0.5 * qq / r;
                    fr += qq / (r * r2);
                }
                for (int k = 0; k < 3; ++k) fi[k] -= fr * d[k];
            }
        });
        for (int k = 0; k < 3; ++k) forces[3 * (size_t)r + k] = fi[k];
    }
    energies[0] = e_lj;
    energies[1] = e_c;
    grid_free(&g);
}

/* ------------------------------------------------------------------------ */
/* Ewald: reciprocal k-sum, exclusion correction, self and net-charge terms */
/* ------------------------------------------------------------------------ */
/*
 * E_rec = k/(2 pi V) sum_{m != 0} exp(-pi^2 m^2/beta^2)/m^2 |S(m)|^2,
 * S(m) = sum_j q_j exp(2 pi i m.r_j), m = (nx/Lx, ny/Ly, nz/Lz), |n_d| <= nmax_d.
 * F_i = (2k/V) q_i sum_m g(m) m Im[exp(2 pi i m.r_i) S*(m)].
 * Sum over the half space (m and -m give equal terms).
 */
double ORC_API orc_ewald_recip(const double *pos, int n, const double *box, const double *q,
                               double beta, const int *nmax, double kcoul, double *forces,
                               const int *subset, int nsub) {
    const int mx = nmax[0], my = nmax[1], mz = nmax[2];
    const double V = box[0] * box[1] * box[2];
    const double pi = 3.14159265358979323846;
    /* per-atom phase tables e^{2 pi i n x/L} for n = 0..nmax (and conj for negative) */
    double *cx = malloc(sizeof(double) * 2 * (size_t)n * (mx + 1));
    double *cy = malloc(sizeof(double) * 2 * (size_t)n * (my + 1));
    double *cz = malloc(sizeof(double) * 2 * (size_t)n * (mz + 1));
    double *tabs[3] = {cx, cy, cz};
    int nm[3] = {mx, my, mz};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        for (int d = 0; d < 3; ++d) {
            double th = 2 * pi * pos[3 * i + d] / box[d];
            double c1 = cos(th), s1 = sin(th);
            double *t = tabs[d] + 2 * (size_t)i * (nm[d] + 1);
            t[0] = 1;
            t[1] = 0;
            for (int k = 1; k <= nm[d]; ++k) {
                /* direct evaluation keeps the tables accurate to ~1 ulp */
                t[2 * k] = cos(th * k);
                t[2 * k + 1] = sin(th * k);
            }
            (void)c1;
            (void)s1;
        }
    }
    /* enumerate half-space m: nx > 0, or nx == 0 && ny > 0, or nx == ny == 0 && nz > 0 */
    long nk = 0;
    for (int a = 0; a <= mx; ++a)
        for (int b = -my; b <= my; ++b)
            for (int c = -mz; c <= mz; ++c) {
                if (a == 0 && (b < 0 || (b == 0 && c <= 0))) continue;
                ++nk;
            }
    int *ks = malloc(sizeof(int) * 3 * nk);
    nk = 0;
    for (int a = 0; a <= mx; ++a)
        for (int b = -my; b <= my; ++b)
            for (int c = -mz; c <= mz; ++c) {
                if (a == 0 && (b < 0 || (b == 0 && c <= 0))) continue;
                ks[3 * nk] = a;
                ks[3 * nk + 1] = b;
                ks[3 * nk + 2] = c;
                ++nk;
            }
    double *Sre = malloc(sizeof(double) * nk), *Sim = malloc(sizeof(double) * nk),
           *gk = malloc(sizeof(double) * nk);
    double energy = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : energy)
    for (long k = 0; k < nk; ++k) {
        int a = ks[3 * k], b = ks[3 * k + 1], c = ks[3 * k + 2];
        double m0 = a / box[0], m1 = b / box[1], m2 = c / box[2];
        double m2sum = m0 * m0 + m1 * m1 + m2 * m2;
        double g = exp(-pi * pi * m2sum / (beta * beta)) / m2sum;
        double sr = 0, si = 0;
        for (int i = 0; i < n; ++i) {
            const double *tx = cx + 2 * ((size_t)i * (mx + 1) + a);
            const double *ty = cy + 2 * ((size_t)i * (my + 1) + abs(b));
            const double *tz = cz + 2 * ((size_t)i * (mz + 1) + abs(c));
            double yr = ty[0], yi = b < 0 ? -ty[1] : ty[1];
            double zr = tz[0], zi = c < 0 ? -tz[1] : tz[1];
            double xyr = tx[0] * yr - tx[1] * yi, xyi = tx[0] * yi + tx[1] * yr;
            double er = xyr * zr - xyi * zi, ei = xyr * zi + xyi * zr;
            sr += q[i] * er;
            si += q[i] * ei;
        }
        Sre[k] = sr;
        Sim[k] = si;
        gk[k] = g;
        energy += 2 * g * (sr * sr + si * si); /* x2: the -m half */
    }
    energy *= kcoul / (2 * pi * V);
    if (forces) {
        /* forces for every atom, or only for the atoms listed in subset
           (written to forces[3*s .. 3*s+2] for the s-th listed atom) */
        const int nout = subset ? nsub : n;
#pragma omp parallel for schedule(static)
        for (int s_ = 0; s_ < nout; ++s_) {
            const int i = subset ? subset[s_] : s_;
            double f[3] = {0, 0, 0};
            for (long k = 0; k < nk; ++k) {
                int a = ks[3 * k], b = ks[3 * k + 1], c = ks[3 * k + 2];
                const double *tx = cx + 2 * ((size_t)i * (mx + 1) + a);
                const double *ty = cy + 2 * ((size_t)i * (my + 1) + abs(b));
                const double *tz = cz + 2 * ((size_t)i * (mz + 1) + abs(c));
                double yr = ty[0], yi = b < 0 ? -ty[1] : ty[1];
                double zr = tz[0], zi = c < 0 ? -tz[1] : tz[1];
                double xyr = tx[0] * yr - tx[1] * yi, xyi = tx[0] * yi + tx[1] * yr;
                double er = xyr * zr - xyi * zi, ei = xyr * zi + xyi * zr;
                /* Im[e_i * conj(S)] */
                double im = ei * Sre[k] - er * Sim[k];
                double w = 2 * gk[k] * im; /* x2: the -m half */
                f[0] += w * a / box[0];
                f[1] += w * b / box[1];
                f[2] += w * c / box[2];
            }
            double pre = 2 * kcoul / V * q[i];
            for (int d = 0; d < 3; ++d) forces[3 * s_ + d] = pre * f[d];
        }
    }
    free(cx);
    free(cy);
    free(cz);
    free(ks);
    free(Sre);
    free(Sim);
    free(gk);
    return energy;
}

/*
 * -k qq erf(beta r)/r for every excluded pair (listed in `excl`, counted once
 * per unordered pair).  Adds into forces, returns the energy.
 */
double ORC_API orc_ewald_exclusions(const double *pos, int n, const double *box, const double *q,
                                    const int *excl, int excl_width, double beta, double kcoul,
                                    double *forces) {
    const double two_over_sqrtpi = 1.1283791670955126;
    double e = 0;
    for (int i = 0; i < n; ++i) {
        for (int w = 0; w < excl_width; ++w) {
            int j = excl[(long)i * excl_width + w];
            if (j <= i) continue;
            double d[3], r2 = 0;
            for (int k = 0; k < 3; ++k) {
                d[k] = wrap1(pos[3 * j + k] - pos[3 * i + k], box[k]);
                r2 += d[k] * d[k];
            }
            double r = sqrt(r2), qq = kcoul * q[i] * q[j];
            double ef = erf(beta * r);
            e -= qq * ef / r;
            /* V = -qq erf(br)/r ; -dV/dr / r = qq (2b/sqrtpi e^{-b^2r^2} r - erf)/r^3 */
            double fr = qq * (beta * two_over_sqrtpi * exp(-beta * beta * r2) * r - ef) / (r2 * r);
            /* force on j = -dV/dr rhat = fr*d */
            for (int k = 0; k < 3; ++k) {
                forces[3 * j + k] += fr * d[k];
                forces[3 * i + k] -= fr * d[k];
            }
        }
    }
    return e;
}

/* ------------------------------------------------------------------------ */
/* PME (FP64): B-spline spread and gather; the FFTs are done by the caller  */
/* ------------------------------------------------------------------------ */
/*
 * Cardinal B-spline weights for fractional offset w in [0,1): on return
 * th[i] = M_p(w + p - 1 - i) and dth[i] = d th[i] / dw, i = 0..p-1, so that
 * grid point floor(u) - p + 1 + i receives weight th[i].  Recursion
 * M_n(x) = x/(n-1) M_{n-1}(x) + (n-x)/(n-1) M_{n-1}(x-1) (Essmann et al. 1995,
 * eqs. 4.1-4.2); the derivative uses M_n'(x) = M_{n-1}(x) - M_{n-1}(x-1).
 */
static void bspline(double w, int order, double *th, double *dth) {
    double a[16];
    memset(a, 0, sizeof(a));
    a[0] = 1 - w; /* order 2: M_2(w+1) */
    a[1] = w;     /*          M_2(w)   */
    for (int n = 3; n <= order; ++n) {
        if (n == order) {
            dth[0] = -a[0];
            for (int i = 1; i < order; ++i) dth[i] = a[i - 1] - a[i];
        }
        double div = 1.0 / (n - 1);
        double b[16];
        /* M_n(w + n-1-i) = ((w+n-1-i) M_{n-1}(w+n-1-i) + (i+1-w) M_{n-1}(w+n-2-i)) / (n-1)
           with M_{n-1}(w + n-2-i') = a[i'] for i' = 0..n-2 */
        for (int i = 0; i < n; ++i) {
            double left = (i >= 1) ? a[i - 1] : 0.0;  /* M_{n-1}(w + n-1-i) */
            double right = (i <= n - 2) ? a[i] : 0.0; /* M_{n-1}(w + n-2-i) */
            b[i] = div * ((w + n - 1 - i) * left + (i + 1 - w) * right);
        }
        for (int i = 0; i < n; ++i) a[i] = b[i];
    }
    if (order == 2) {
        dth[0] = -1;
        dth[1] = 1;
    }
    for (int i = 0; i < order; ++i) th[i] = a[i];
}

/*
 * Spread q onto a K0*K1*K2 real grid (row-major, index (g0*K1+g1)*K2+g2).
 * u_d = K_d * x_d / L_d; m = floor(u); w = u - m; atom weight theta[k] lands on
 * grid point (m - order + 1 + k) mod K (k = 0..order-1).
 */
void ORC_API orc_pme_spread(const double *pos, int n, const double *box, const double *q,
                            const int *K, int order, double *grid) {
    long tot = (long)K[0] * K[1] * K[2];
    memset(grid, 0, sizeof(double) * tot);
    for (int i = 0; i < n; ++i) {
        double th[3][16], dth[3][16];
        int m0[3];
        for (int d = 0; d < 3; ++d) {
            double u = pos[3 * i + d] / box[d];
            u = (u - floor(u)) * K[d];
            int m = (int)floor(u);
            double w = u - m;
            bspline(w, order, th[d], dth[d]);
            m0[d] = m - order + 1;
        }
        for (int a = 0; a < order; ++a) {
            int ga = ((m0[0] + a) % K[0] + K[0]) % K[0];
            for (int b = 0; b < order; ++b) {
                int gb = ((m0[1] + b) % K[1] + K[1]) % K[1];
                double wab = q[i] * th[0][a] * th[1][b];
                for (int c = 0; c < order; ++c) {
                    int gc = ((m0[2] + c) % K[2] + K[2]) % K[2];
                    grid[((long)ga * K[1] + gb) * K[2] + gc] += wab * th[2][c];
                }
            }
        }
    }
}

/* forces F_i = -q_i sum grad(theta) phi, grad in x: dtheta * K/L */
void ORC_API orc_pme_gather(const double *pos, int n, const double *box, const double *q,
                            const int *K, int order, const double *phi, double scale,
                            double *forces) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double th[3][16], dth[3][16];
        int m0[3];
        for (int d = 0; d < 3; ++d) {
            double u = pos[3 * i + d] / box[d];
            u = (u - floor(u)) * K[d];
            int m = (int)floor(u);
            double w = u - m;
            bspline(w, order, th[d], dth[d]);
            m0[d] = m - order + 1;
        }
        double f[3] = {0, 0, 0};
        for (int a = 0; a < order; ++a) {
            int ga = ((m0[0] + a) % K[0] + K[0]) % K[0];
            double ta = th[0][a], da = dth[0][a];
            for (int b = 0; b < order; ++b) {
                int gb = ((m0[1] + b) % K[1] + K[1]) % K[1];
                double tb = th[1][b], db = dth[1][b];
                for (int c = 0; c < order; ++c) {
                    int gc = ((m0[2] + c) % K[2] + K[2]) % K[2];
                    double tc = th[2][c], dc = dth[2][c];
                    double p = phi[((long)ga * K[1] + gb) * K[2] + gc];
                    f[0] += da * tb * tc * p;
                    f[1] += ta * db * tc * p;
                    f[2] += ta * tb * dc * p;
                }
            }
        }
        for (int d = 0; d < 3; ++d) forces[3 * i + d] = -scale * q[i] * f[d] * K[d] / box[d];
    }
}

/* B-spline moduli |b(m)|^2 for one dimension (Essmann et al. 1995, eq. 4.4) */
void ORC_API orc_bspline_moduli(int K, int order, double *mod) {
    double th[16], dth[16];
    bspline(0.0, order, th, dth);
    /* M_p(k+1) for k = 0..p-2 equals th[...] at w = 0 */
    const double pi = 3.14159265358979323846;
    for (int m = 0; m < K; ++m) {
        double sr = 0, si = 0;
        for (int k = 0; k <= order - 2; ++k) {
            double mk = th[order - 2 - k]; /* th[i] = M_p(p-1-i) at w = 0 */
            double arg = 2 * pi * m * k / K;
            sr += mk * cos(arg);
            si += mk * sin(arg);
        }
        mod[m] = sr * sr + si * si;
    }
    /* guard zeros (odd order at Nyquist) by neighbour averaging */
    for (int m = 0; m < K; ++m)
        if (mod[m] < 1e-10) mod[m] = 0.5 * (mod[(m - 1 + K) % K] + mod[(m + 1) % K]);
}

/* ------------------------------------------------------------------------ */
/* bonded terms (FP64, exact gradients)                                     */
/* ------------------------------------------------------------------------ */
static inline void mi(const double *pos, const double *box, int a, int b, double *d) {
    for (int k = 0; k < 3; ++k) d[k] = wrap1(pos[3 * b + k] - pos[3 * a + k], box[k]);
}
static inline double dot3(const double *a, const double *b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

/* V = k (r - r0)^2  (charmm_bond_constraint.py:57-72) */
double ORC_API orc_bonds(const double *pos, const double *box, const int *idx, const double *prm,
                         int nb, double *forces) {
    double e = 0;
    for (int t = 0; t < nb; ++t) {
        int i = idx[2 * t], j = idx[2 * t + 1];
        double d[3];
        mi(pos, box, i, j, d);
        double r = sqrt(dot3(d, d)), k = prm[2 * t], r0 = prm[2 * t + 1];
        e += k * (r - r0) * (r - r0);
        double f = 2 * k * (r - r0) / r; /* pulls j toward i when stretched */
        for (int c = 0; c < 3; ++c) {
            forces[3 * i + c] += f * d[c];
            forces[3 * j + c] -= f * d[c];
        }
    }
    return e;
}

/* V = k (theta - theta0)^2 + ku (r13 - u0)^2  (charmm_angle_constraint.py:143-178) */
double ORC_API orc_angles(const double *pos, const double *box, const int *idx, const double *prm,
                          int na, double *forces) {
    double e = 0;
    for (int t = 0; t < na; ++t) {
        int i = idx[3 * t], j = idx[3 * t + 1], l = idx[3 * t + 2];
        double k = prm[4 * t], th0 = prm[4 * t + 1], ku = prm[4 * t + 2], u0 = prm[4 * t + 3];
        double a[3], b[3];
        mi(pos, box, j, i, a); /* r21 = x_i - x_j */
        mi(pos, box, j, l, b); /* r23 = x_l - x_j */
        double la = sqrt(dot3(a, a)), lb = sqrt(dot3(b, b));
        double c = dot3(a, b) / (la * lb);
        if (c > 1) c = 1;
        if (c < -1) c = -1;
        double th = acos(c), s = sqrt(1 - c * c);
        if (s < 1e-12) s = 1e-12;
        e += k * (th - th0) * (th - th0);
        double dvdth = 2 * k * (th - th0);
        /* dtheta/dx_i = -(b/(la lb) - c a/la^2)/s */
        for (int q = 0; q < 3; ++q) {
            double dti = -(b[q] / (la * lb) - c * a[q] / (la * la)) / s;
            double dtl = -(a[q] / (la * lb) - c * b[q] / (lb * lb)) / s;
            forces[3 * i + q] -= dvdth * dti;
            forces[3 * l + q] -= dvdth * dtl;
            forces[3 * j + q] += dvdth * (dti + dtl);
        }
        if (ku != 0) {
            double d[3];
            mi(pos, box, i, l, d);
            double r = sqrt(dot3(d, d));
            e += ku * (r - u0) * (r - u0);
            double f = 2 * ku * (r - u0) / r;
            for (int q = 0; q < 3; ++q) {
                forces[3 * i + q] += f * d[q];
                forces[3 * l + q] -= f * d[q];
            }
        }
    }
    return e;
}

/* dihedral angle as get_pbc_dihedral (mdpy/utils/geometry.py:73-86) and its gradient */
static double torsion(const double *pos, const double *box, int i, int j, int k, int l,
                      double g[4][3]) {
    double b1[3], b2[3], b3[3], m[3], nn[3];
    mi(pos, box, i, j, b1);
    mi(pos, box, j, k, b2);
    mi(pos, box, k, l, b3);
    cross3(b1, b2, m);
    cross3(b2, b3, nn);
    double lb2 = sqrt(dot3(b2, b2));
    double x = lb2 * dot3(b1, nn), y = dot3(m, nn);
    double phi = atan2(x, y);
    double m2 = dot3(m, m), n2 = dot3(nn, nn);
    for (int q = 0; q < 3; ++q) {
        g[0][q] = -lb2 / m2 * m[q];
        g[3][q] = lb2 / n2 * nn[q];
    }
    /* Blondel & Karplus, J. Comput. Chem. 17 (1996) 1132, in bond-vector form:
       p = b1.b2/|b2|^2, r = b3.b2/|b2|^2 */
    double p = dot3(b1, b2) / (lb2 * lb2), r = dot3(b3, b2) / (lb2 * lb2);
    for (int q = 0; q < 3; ++q) {
        g[1][q] = -(1 + p) * g[0][q] + r * g[3][q];
        g[2][q] = p * g[0][q] - (1 + r) * g[3][q];
    }
    return phi;
}

/* V = k (1 + cos(n phi - delta)); prm rows (k, n, delta) */
double ORC_API orc_dihedrals(const double *pos, const double *box, const int *idx,
                             const double *prm, int nd, double *forces) {
    double e = 0;
    for (int t = 0; t < nd; ++t) {
        double g[4][3];
        int id[4] = {idx[4 * t], idx[4 * t + 1], idx[4 * t + 2], idx[4 * t + 3]};
        double phi = torsion(pos, box, id[0], id[1], id[2], id[3], g);
        double k = prm[3 * t], nm = prm[3 * t + 1], dl = prm[3 * t + 2];
        e += k * (1 + cos(nm * phi - dl));
        double dv = -k * nm * sin(nm * phi - dl);
        for (int a = 0; a < 4; ++a)
            for (int q = 0; q < 3; ++q) forces[3 * id[a] + q] -= dv * g[a][q];
    }
    return e;
}

/* V = k (psi - psi0)^2; prm rows (k, psi0) */
double ORC_API orc_impropers(const double *pos, const double *box, const int *idx,
                             const double *prm, int ni, double *forces) {
    const double pi = 3.14159265358979323846;
    double e = 0;
    for (int t = 0; t < ni; ++t) {
        double g[4][3];
        int id[4] = {idx[4 * t], idx[4 * t + 1], idx[4 * t + 2], idx[4 * t + 3]};
        double psi = torsion(pos, box, id[0], id[1], id[2], id[3], g);
        double k = prm[2 * t], p0 = prm[2 * t + 1];
        double dp = psi - p0;
        if (dp > pi) dp -= 2 * pi;
        if (dp < -pi) dp += 2 * pi;
        e += k * dp * dp;
        double dv = 2 * k * dp;
        for (int a = 0; a < 4; ++a)
            for (int q = 0; q < 3; ++q) forces[3 * id[a] + q] -= dv * g[a][q];
    }
    return e;
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 and the thermostat noise                                    */
/* ------------------------------------------------------------------------ */
static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

void ORC_API orc_philox4x32(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
        mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/*
 * Three N(0,1) numbers per atom for integrator step `step`:
 * counter (atom, step_lo, step_hi, 0x4C414E47 "LANG"), key = seed (lo, hi);
 * u_k = ((x_k >> 8) + 0.5) * 2^-24 in float32; Box-Muller in float32:
 * g0 = sqrt(-2 ln u0) cos(2 pi u1), g1 = sqrt(-2 ln u0) sin(2 pi u1),
 * g2 = sqrt(-2 ln u2) cos(2 pi u3).
 */
void ORC_API orc_langevin_noise(int n, uint64_t seed, uint64_t step, float *out) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int i = 0; i < n; ++i) {
        uint32_t ctr[4] = {(uint32_t)i, (uint32_t)step, (uint32_t)(step >> 32), 0x4C414E47u};
        uint32_t x[4];
        orc_philox4x32(ctr, key, x);
        float u[4];
        for (int k = 0; k < 4; ++k) u[k] = ((float)(x[k] >> 8) + 0.5f) * 5.9604644775390625e-8f;
        float r0 = sqrtf(-2.0f * logf(u[0])), r1 = sqrtf(-2.0f * logf(u[2]));
        const float twopi = 6.28318530717958647692f;
        out[3 * i] = r0 * cosf(twopi * u[1]);
        out[3 * i + 1] = r0 * sinf(twopi * u[1]);
        out[3 * i + 2] = r1 * cosf(twopi * u[3]);
    }
}
