/*
 * ORACLE - test infrastructure only.  Nothing in the product links, loads or
 * calls this file; it is the CPU checker that the tests, smoke() and the
 * bench's CPU-baseline leg use.
 *
 * Plain-C FP64 restatement of the single-wall Rotne-Prager-Yamakawa blob
 * mobility products of RigidMultiblobsWall:
 *
 *   kind 0  u = M_UF f   mobility/mobility_numba.py:124-287   (1/(8 pi eta a))
 *   kind 1  u = M_UT t   mobility/mobility_numba.py:548-686   (1/(8 pi eta a^2))
 *   kind 2  w = M_WF f   mobility/mobility_numba.py:938-1073  (1/(8 pi eta a^2))
 *   kind 3  w = M_WT t   mobility/mobility_numba.py:1189-1328 (1/(8 pi eta a^3))
 *
 * The expressions keep the reference's operation order so that, compiled
 * without fast-math and without FMA contraction, the results match the
 * reference's own Python/numba source to round-off.  Periodic images follow
 * the numba source: x/y/z minimum-image projection plus the +-1 neighbour
 * boxes when L[k] > 0; the wall term always uses (z_i + z_j)/a (unprojected).
 *
 * oracle_wall_product adds the wall regularisation of mobility/mobility.py:52-84
 * (z_eff = max(z, a) when z <= a; B = diag(min(z/a, 1)) when z < a; the product
 * is B M(z_eff) B v) exactly like the *_numba wrappers (mobility/mobility.py:1132-1341).
 *
 * oracle_wall_uf_symmetric restates the loop structure of the reference's C++
 * product (mobility/mobility.cpp:256-430): OpenMP over targets, only pairs
 * j > i are evaluated and M_ij^T f_i is scattered to u_j (the wall mobility is
 * symmetric), per-thread private accumulators reduced at the end.  It is the
 * timed CPU baseline (non-periodic only).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double PI_ = 3.14159265358979323846;

static double project(double d, double L)
{
    /* rx = rx - int(rx / L + 0.5 * (int(rx>0) - int(rx<0))) * L */
    double s = (double)((d > 0) - (d < 0));
    return d - (double)(long)(d / L + 0.5 * s) * L;
}

/* One 3x3 block of the (unregularised) wall mobility times v_j, accumulated
 * into acc[3].  (rx, ry, rz) = (r_i - r_j) after periodic projection and image
 * shift, unscaled.  self != 0 selects the i == j (central box) branch. */
static void pair_block(int kind, double rx, double ry, double rz,
                       double zi, double zj, int self, double inva,
                       const double *vj, double *acc)
{
    double Mxx, Mxy, Mxz, Myx, Myy, Myz, Mzx, Mzy, Mzz;
    const double fourOverThree = 4.0 / 3.0;
    rx *= inva;
    ry *= inva;
    rz *= inva;
    if (kind == 0) {
        if (self) {
            Mxx = fourOverThree; Mxy = 0; Mxz = 0; Myy = Mxx; Myz = 0; Mzz = Mxx;
        } else {
            double r2 = rx * rx + ry * ry + rz * rz;
            double r = sqrt(r2);
            double invr = 1.0 / r;
            double invr2 = invr * invr;
            double c1, c2;
            if (r > 2) {
                c1 = 1.0 + 2.0 / (3.0 * r2);
                c2 = (1.0 - 2.0 * invr2) * invr2;
                Mxx = (c1 + c2 * rx * rx) * invr;
                Mxy = (c2 * rx * ry) * invr;
                Mxz = (c2 * rx * rz) * invr;
                Myy = (c1 + c2 * ry * ry) * invr;
                Myz = (c2 * ry * rz) * invr;
                Mzz = (c1 + c2 * rz * rz) * invr;
            } else {
                c1 = fourOverThree * (1.0 - 0.28125 * r);
                c2 = fourOverThree * 0.09375 * invr;
                Mxx = c1 + c2 * rx * rx;
                Mxy = c2 * rx * ry;
                Mxz = c2 * rx * rz;
                Myy = c1 + c2 * ry * ry;
                Myz = c2 * ry * rz;
                Mzz = c1 + c2 * rz * rz;
            }
        }
        Myx = Mxy; Mzx = Mxz; Mzy = Myz;
        double Rz = (zi + zj) * inva;
        double hj = zj * inva;
        if (self) {
            double invZi = 1.0 / hj;
            double invZi3 = invZi * invZi * invZi;
            double invZi5 = invZi3 * invZi * invZi;
            Mxx += -(9.0 * invZi - 2.0 * invZi3 + invZi5) / 12.0;
            Myy += -(9.0 * invZi - 2.0 * invZi3 + invZi5) / 12.0;
            Mzz += -(9.0 * invZi - 4.0 * invZi3 + invZi5) / 6.0;
        } else {
            double h_hat = hj / Rz;
            double invR = 1.0 / sqrt(rx * rx + ry * ry + Rz * Rz);
            double ex = rx * invR, ey = ry * invR, ez = Rz * invR;
            double invR3 = invR * invR * invR;
            double invR5 = invR3 * invR * invR;
            double fact1 = -(3.0 * (1.0 + 2.0 * h_hat * (1.0 - h_hat) * ez * ez) * invR + 2.0 * (1.0 - 3.0 * ez * ez) * invR3 - 2.0 * (1.0 - 5.0 * ez * ez) * invR5) / 3.0;
            double fact2 = -(3.0 * (1.0 - 6.0 * h_hat * (1.0 - h_hat) * ez * ez) * invR - 6.0 * (1.0 - 5.0 * ez * ez) * invR3 + 10.0 * (1.0 - 7.0 * ez * ez) * invR5) / 3.0;
            double fact3 = ez * (3.0 * h_hat * (1.0 - 6.0 * (1.0 - h_hat) * ez * ez) * invR - 6.0 * (1.0 - 5.0 * ez * ez) * invR3 + 10.0 * (2.0 - 7.0 * ez * ez) * invR5) * 2.0 / 3.0;
            double fact4 = ez * (3.0 * h_hat * invR - 10.0 * invR5) * 2.0 / 3.0;
            double fact5 = -(3.0 * h_hat * h_hat * ez * ez * invR + 3.0 * ez * ez * invR3 + (2.0 - 15.0 * ez * ez) * invR5) * 4.0 / 3.0;
            Mxx += fact1 + fact2 * ex * ex;
            Mxy += fact2 * ex * ey;
            Mxz += fact2 * ex * ez + fact3 * ex;
            Myx += fact2 * ey * ex;
            Myy += fact1 + fact2 * ey * ey;
            Myz += fact2 * ey * ez + fact3 * ey;
            Mzx += fact2 * ez * ex + fact4 * ex;
            Mzy += fact2 * ez * ey + fact4 * ey;
            Mzz += fact1 + fact2 * ez * ez + fact3 * ez + fact4 * ez + fact5;
        }
    } else if (kind == 1 || kind == 2) {
        /* RPY rotation-translation coupling (same for UT and WF). */
        if (self) {
            Mxx = 0; Mxy = 0; Mxz = 0; Myy = 0; Myz = 0; Mzz = 0;
        } else {
            double r2 = rx * rx + ry * ry + rz * rz;
            double r = sqrt(r2);
            double r3 = r2 * r;
            double invr3 = 1.0 / r3;
            if (r >= 2) {
                Mxx = 0; Mxy = rz * invr3; Mxz = -ry * invr3;
                Myy = 0; Myz = rx * invr3; Mzz = 0;
            } else {
                double c1 = 0.5 * (1.0 - 0.375 * r);
                Mxx = 0; Mxy = c1 * rz; Mxz = -c1 * ry;
                Myy = 0; Myz = c1 * rx; Mzz = 0;
            }
        }
        Myx = -Mxy; Mzx = -Mxz; Mzy = -Myz;
        if (kind == 1) {
            /* UT: wall term with i and j swapped (mobility_numba.py:646-651). */
            double sx = -rx, sy = -ry;
            double Rz = (zi + zj) * inva;
            double hj = zi * inva;
            if (self) {
                double invZi = 1.0 / hj;
                double invZi4 = invZi * invZi * invZi * invZi;
                Mxy -= -invZi4 * 0.125;
                Myx -= invZi4 * 0.125;
            } else {
                double h_hat = hj / Rz;
                double invR = 1.0 / sqrt(sx * sx + sy * sy + Rz * Rz);
                double invR2 = invR * invR;
                double invR4 = invR2 * invR2;
                double ex = sx * invR, ey = sy * invR, ez = Rz * invR;
                double fact1 = invR2;
                double fact2 = (6.0 * h_hat * ez * ez * invR2 + (1.0 - 10.0 * ez * ez) * invR4) * 2.0;
                double fact3 = -ez * (3.0 * h_hat * invR2 - 5.0 * invR4) * 2.0;
                double fact4 = -ez * (h_hat * invR2 - invR4) * 2.0;
                Mxx -= -fact3 * ex * ey;
                Mxy -= -fact1 * ez + fact3 * ex * ex - fact4;
                Mxz -= fact1 * ey;
                Myx -= fact1 * ez - fact3 * ey * ey + fact4;
                Myy -= fact3 * ex * ey;
                Myz -= -fact1 * ex;
                Mzx -= -fact1 * ey - fact2 * ey - fact3 * ey * ez;
                Mzy -= fact1 * ex + fact2 * ex + fact3 * ex * ez;
            }
        } else {
            /* WF */
            double Rz = (zi + zj) * inva;
            double hj = zj * inva;
            if (self) {
                double invZi = 1.0 / hj;
                double invZi4 = invZi * invZi * invZi * invZi;
                Mxy += -invZi4 * 0.125;
                Myx += invZi4 * 0.125;
            } else {
                double h_hat = hj / Rz;
                double invR = 1.0 / sqrt(rx * rx + ry * ry + Rz * Rz);
                double invR2 = invR * invR;
                double invR4 = invR2 * invR2;
                double ex = rx * invR, ey = ry * invR, ez = Rz * invR;
                double fact1 = invR2;
                double fact2 = (6.0 * h_hat * ez * ez * invR2 + (1.0 - 10.0 * ez * ez) * invR4) * 2.0;
                double fact3 = -ez * (3.0 * h_hat * invR2 - 5.0 * invR4) * 2.0;
                double fact4 = -ez * (h_hat * invR2 - invR4) * 2.0;
                Mxx -= -fact3 * ex * ey;
                Mxy -= fact1 * ez - fact3 * ey * ey + fact4;
                Mxz -= -fact1 * ey - fact2 * ey - fact3 * ey * ez;
                Myx -= -fact1 * ez + fact3 * ex * ex - fact4;
                Myy -= fact3 * ex * ey;
                Myz -= fact1 * ex + fact2 * ex + fact3 * ex * ez;
                Mzx -= fact1 * ey;
                Mzy -= -fact1 * ex;
            }
        }
    } else {
        /* kind 3: WT */
        if (self) {
            Mxx = 1.0; Mxy = 0; Mxz = 0; Myy = Mxx; Myz = 0; Mzz = Mxx;
        } else {
            double r2 = rx * rx + ry * ry + rz * rz;
            double r = sqrt(r2);
            double r3 = r2 * r;
            double invr = 1.0 / r;
            double invr2 = 1.0 / r2;
            double invr3 = 1.0 / r3;
            if (r >= 2) {
                double c1 = -0.5;
                double c2 = 1.5 * invr2;
                Mxx = (c1 + c2 * rx * rx) * invr3;
                Mxy = (c2 * rx * ry) * invr3;
                Mxz = (c2 * rx * rz) * invr3;
                Myy = (c1 + c2 * ry * ry) * invr3;
                Myz = (c2 * ry * rz) * invr3;
                Mzz = (c1 + c2 * rz * rz) * invr3;
            } else {
                double c1 = (1.0 - 0.84375 * r + 0.078125 * r3);
                double c2 = 0.28125 * invr - 0.046875 * r;
                Mxx = c1 + c2 * rx * rx;
                Mxy = c2 * rx * ry;
                Mxz = c2 * rx * rz;
                Myy = c1 + c2 * ry * ry;
                Myz = c2 * ry * rz;
                Mzz = c1 + c2 * rz * rz;
            }
        }
        Myx = Mxy; Mzx = Mxz; Mzy = Myz;
        double Rz = (zi + zj) * inva;
        double hj = zj * inva;
        if (self) {
            double invZi = 1.0 / hj;
            double invZi3 = invZi * invZi * invZi;
            Mxx += -invZi3 * 0.3125;
            Myy += -invZi3 * 0.3125;
            Mzz += -invZi3 * 0.125;
        } else {
            double invR = 1.0 / sqrt(rx * rx + ry * ry + Rz * Rz);
            double invR3 = invR * invR * invR;
            double ex = rx * invR, ey = ry * invR, ez = Rz * invR;
            double fact1 = ((1.0 - 6.0 * ez * ez) * invR3) * 0.5;
            double fact2 = -(9.0 * invR3) / 6.0;
            double fact3 = (3.0 * invR3 * ez);
            double fact4 = (3.0 * invR3);
            Mxx += fact1 + fact2 * ex * ex + fact4 * ey * ey;
            Mxy += (fact2 - fact4) * ex * ey;
            Mxz += fact2 * ex * ez;
            Myx += (fact2 - fact4) * ex * ey;
            Myy += fact1 + fact2 * ey * ey + fact4 * ex * ex;
            Myz += fact2 * ey * ez;
            Mzx += fact2 * ez * ex + fact3 * ex;
            Mzy += fact2 * ez * ey + fact3 * ey;
            Mzz += fact1 + fact2 * ez * ez + fact3 * ez;
        }
    }
    acc[0] += Mxx * vj[0] + Mxy * vj[1] + Mxz * vj[2];
    acc[1] += Myx * vj[0] + Myy * vj[1] + Myz * vj[2];
    acc[2] += Mzx * vj[0] + Mzy * vj[1] + Mzz * vj[2];
}

static double norm_factor(int kind, double eta, double a)
{
    double p = (kind == 0) ? a : (kind == 3 ? a * a * a : a * a);
    return 1.0 / (8.0 * PI_ * eta * p);
}

/* out[3*t..3*t+2] for targets rows[t] (or all targets when rows == NULL);
 * positions r are used as given (no wall regularisation). */
void oracle_wall_raw_rows(int kind, const double *r, const double *v, double *out,
                          long n, const long *rows, long nrows,
                          double eta, double a, const double *L)
{
    double Lx = L ? L[0] : 0.0, Ly = L ? L[1] : 0.0, Lz = L ? L[2] : 0.0;
    int px = Lx > 0, py = Ly > 0, pz = Lz > 0;
    double inva = 1.0 / a;
    double nf = norm_factor(kind, eta, a);
    long nt = rows ? nrows : n;
#pragma omp parallel for schedule(dynamic, 16)
    for (long t = 0; t < nt; ++t) {
        long i = rows ? rows[t] : t;
        double acc[3] = {0.0, 0.0, 0.0};
        for (int bx = -px; bx <= px; ++bx)
            for (int by = -py; by <= py; ++by)
                for (int bz = -pz; bz <= pz; ++bz)
                    for (long j = 0; j < n; ++j) {
                        double rx = r[3 * i] - r[3 * j];
                        double ry = r[3 * i + 1] - r[3 * j + 1];
                        double rz = r[3 * i + 2] - r[3 * j + 2];
                        if (Lx > 0) rx = project(rx, Lx) + bx * Lx;
                        if (Ly > 0) ry = project(ry, Ly) + by * Ly;
                        if (Lz > 0) rz = project(rz, Lz) + bz * Lz;
                        int self = (i == j) && bx == 0 && by == 0 && bz == 0;
                        /* Each block's product is scaled by the norm factor
                         * before accumulation, as in the reference. */
                        double blk[3] = {0.0, 0.0, 0.0};
                        pair_block(kind, rx, ry, rz, r[3 * i + 2], r[3 * j + 2], self, inva, v + 3 * j, blk);
                        acc[0] += blk[0] * nf;
                        acc[1] += blk[1] * nf;
                        acc[2] += blk[2] * nf;
                    }
        out[3 * t] = acc[0];
        out[3 * t + 1] = acc[1];
        out[3 * t + 2] = acc[2];
    }
}

/* Free-space RPY block (no wall) applied to v, unscaled: the no-wall numba
 * products mobility/mobility_numba.py:13-130 (UF), 440-560 (UT), 832-950 (WF),
 * 1077-1190 (WT), same operation order.  r* are unscaled differences. */
static void rpy_block(int kind, double rx, double ry, double rz, int self, double inva, const double *v,
                      double *out)
{
    double Mxx, Mxy, Mxz, Myy, Myz, Mzz, Myx, Mzx, Mzy;
    if (self) {
        double d = (kind == 0) ? 4.0 / 3.0 : (kind == 3 ? 1.0 : 0.0);
        Mxx = d; Myy = d; Mzz = d;
        Mxy = Mxz = Myz = 0.0;
        Myx = Mzx = Mzy = 0.0;
    } else {
        rx *= inva;
        ry *= inva;
        rz *= inva;
        double r2 = rx * rx + ry * ry + rz * rz;
        double r = sqrt(r2);
        if (kind == 0) {
            double invr = 1.0 / r, invr2 = invr * invr, c1, c2;
            if (r > 2) {
                c1 = 1.0 + 2.0 / (3.0 * r2);
                c2 = (1.0 - 2.0 * invr2) * invr2;
                Mxx = (c1 + c2 * rx * rx) * invr; Mxy = (c2 * rx * ry) * invr; Mxz = (c2 * rx * rz) * invr;
                Myy = (c1 + c2 * ry * ry) * invr; Myz = (c2 * ry * rz) * invr; Mzz = (c1 + c2 * rz * rz) * invr;
            } else {
                c1 = 4.0 / 3.0 * (1.0 - 0.28125 * r);
                c2 = 4.0 / 3.0 * 0.09375 * invr;
                Mxx = c1 + c2 * rx * rx; Mxy = c2 * rx * ry; Mxz = c2 * rx * rz;
                Myy = c1 + c2 * ry * ry; Myz = c2 * ry * rz; Mzz = c1 + c2 * rz * rz;
            }
            Myx = Mxy; Mzx = Mxz; Mzy = Myz;
        } else if (kind == 1 || kind == 2) {
            double r3 = r2 * r, invr3 = 1.0 / r3;
            Mxx = Myy = Mzz = 0.0;
            if (r >= 2) {
                Mxy = rz * invr3; Mxz = -ry * invr3; Myz = rx * invr3;
            } else {
                double c1 = 0.5 * (1.0 - 0.375 * r);
                Mxy = c1 * rz; Mxz = -c1 * ry; Myz = c1 * rx;
            }
            Myx = -Mxy; Mzx = -Mxz; Mzy = -Myz;
        } else {
            double r3 = r2 * r, invr = 1.0 / r, invr2 = 1.0 / r2, invr3 = 1.0 / r3, c1, c2;
            if (r >= 2) {
                c1 = -0.5;
                c2 = 1.5 * invr2;
                Mxx = (c1 + c2 * rx * rx) * invr3; Mxy = (c2 * rx * ry) * invr3; Mxz = (c2 * rx * rz) * invr3;
                Myy = (c1 + c2 * ry * ry) * invr3; Myz = (c2 * ry * rz) * invr3; Mzz = (c1 + c2 * rz * rz) * invr3;
            } else {
                c1 = (1.0 - 0.84375 * r + 0.078125 * r3);
                c2 = 0.28125 * invr - 0.046875 * r;
                Mxx = c1 + c2 * rx * rx; Mxy = c2 * rx * ry; Mxz = c2 * rx * rz;
                Myy = c1 + c2 * ry * ry; Myz = c2 * ry * rz; Mzz = c1 + c2 * rz * rz;
            }
            Myx = Mxy; Mzx = Mxz; Mzy = Myz;
        }
    }
    out[0] = Mxx * v[0] + Mxy * v[1] + Mxz * v[2];
    out[1] = Myx * v[0] + Myy * v[1] + Myz * v[2];
    out[2] = Mzx * v[0] + Mzy * v[1] + Mzz * v[2];
}

/* Free-space RPY product (no wall, no regularisation) for all targets or the
 * listed rows; periodic images as in the wall products. */
void oracle_nowall_rows(int kind, const double *r, const double *v, double *out, long n, const long *rows,
                        long nrows, double eta, double a, const double *L)
{
    double Lx = L ? L[0] : 0.0, Ly = L ? L[1] : 0.0, Lz = L ? L[2] : 0.0;
    int px = Lx > 0, py = Ly > 0, pz = Lz > 0;
    double inva = 1.0 / a;
    double nf = norm_factor(kind, eta, a);
    long nt = rows ? nrows : n;
#pragma omp parallel for schedule(dynamic, 16)
    for (long t = 0; t < nt; ++t) {
        long i = rows ? rows[t] : t;
        double acc[3] = {0.0, 0.0, 0.0};
        for (int bx = -px; bx <= px; ++bx)
            for (int by = -py; by <= py; ++by)
                for (int bz = -pz; bz <= pz; ++bz)
                    for (long j = 0; j < n; ++j) {
                        double rx = r[3 * i] - r[3 * j];
                        double ry = r[3 * i + 1] - r[3 * j + 1];
                        double rz = r[3 * i + 2] - r[3 * j + 2];
                        if (Lx > 0) rx = project(rx, Lx) + bx * Lx;
                        if (Ly > 0) ry = project(ry, Ly) + by * Ly;
                        if (Lz > 0) rz = project(rz, Lz) + bz * Lz;
                        int self = (i == j) && bx == 0 && by == 0 && bz == 0;
                        double blk[3];
                        rpy_block(kind, rx, ry, rz, self, inva, v + 3 * j, blk);
                        acc[0] += blk[0] * nf;
                        acc[1] += blk[1] * nf;
                        acc[2] += blk[2] * nf;
                    }
        out[3 * t] = acc[0];
        out[3 * t + 1] = acc[1];
        out[3 * t + 2] = acc[2];
    }
}

void oracle_wall_raw(int kind, const double *r, const double *v, double *out,
                     long n, double eta, double a, const double *L)
{
    oracle_wall_raw_rows(kind, r, v, out, n, NULL, 0, eta, a, L);
}

/* Wall-regularised product B M(z_eff) B v for all targets, or for the target
 * rows listed in `rows` (out then has 3*nrows entries). */
void oracle_wall_product_rows(int kind, const double *r, const double *v, double *out,
                              long n, const long *rows, long nrows,
                              double eta, double a, const double *L)
{
    double *reff = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    double *vb = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    for (long k = 0; k < n; ++k) {
        double z = r[3 * k + 2];
        double b = (z < a) ? z / a : 1.0;
        reff[3 * k] = r[3 * k];
        reff[3 * k + 1] = r[3 * k + 1];
        reff[3 * k + 2] = (z <= a) ? a : z;
        vb[3 * k] = v[3 * k] * b;
        vb[3 * k + 1] = v[3 * k + 1] * b;
        vb[3 * k + 2] = v[3 * k + 2] * b;
    }
    oracle_wall_raw_rows(kind, reff, vb, out, n, rows, nrows, eta, a, L);
    long nt = rows ? nrows : n;
    for (long t = 0; t < nt; ++t) {
        long i = rows ? rows[t] : t;
        double z = r[3 * i + 2];
        double b = (z < a) ? z / a : 1.0;
        out[3 * t] *= b;
        out[3 * t + 1] *= b;
        out[3 * t + 2] *= b;
    }
    free(reff);
    free(vb);
}

void oracle_wall_product(int kind, const double *r, const double *v, double *out,
                         long n, double eta, double a, const double *L)
{
    oracle_wall_product_rows(kind, r, v, out, n, NULL, 0, eta, a, L);
}

/* Dense wall mobility (3n x 3n, row-major) of n blobs, regularised like
 * single_wall_fluid_mobility (mobility/mobility.py:1018-1116): entries of
 * B M(z_eff) B with the per-pair formulas of the UF product. */
void oracle_wall_dense(const double *r, long n, double eta, double a, double *M)
{
    double inva = 1.0 / a;
    double nf = norm_factor(0, eta, a);
#pragma omp parallel for schedule(dynamic, 4)
    for (long i = 0; i < n; ++i) {
        double zi = r[3 * i + 2];
        double bi = (zi < a) ? zi / a : 1.0;
        double zie = (zi <= a) ? a : zi;
        for (long j = 0; j < n; ++j) {
            double zj = r[3 * j + 2];
            double bj = (zj < a) ? zj / a : 1.0;
            double zje = (zj <= a) ? a : zj;
            for (int c = 0; c < 3; ++c) {
                double e[3] = {0.0, 0.0, 0.0};
                double col[3] = {0.0, 0.0, 0.0};
                e[c] = 1.0;
                pair_block(0, r[3 * i] - r[3 * j], r[3 * i + 1] - r[3 * j + 1], zie - zje, zie, zje, i == j, inva,
                           e, col);
                for (int u = 0; u < 3; ++u) M[(3 * i + u) * 3 * n + 3 * j + c] = col[u] * nf * bi * bj;
            }
        }
    }
}

/* Symmetric-pair M_UF f in the loop structure of mobility/mobility.cpp:256-430
 * (non-periodic).  r must already hold z_eff and f must already be damped. */
void oracle_wall_uf_symmetric(const double *r, const double *f, double *u,
                              long n, double eta, double a, int nthreads)
{
    const double inva = 1.0 / a;
    const double nf = 1.0 / (8.0 * PI_ * eta * a);
    const double fourOverThree = 4.0 / 3.0;
    memset(u, 0, sizeof(double) * 3 * (size_t)n);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        double *up = (double *)calloc(3 * (size_t)n, sizeof(double));
#pragma omp for schedule(dynamic)
        for (long i = 0; i < n; ++i) {
            {
                double invZi = a / r[3 * i + 2];
                double invZi3 = invZi * invZi * invZi;
                double invZi5 = invZi3 * invZi * invZi;
                double Mxx = fourOverThree - (9.0 * invZi - 2.0 * invZi3 + invZi5) / 12.0;
                double Mzz = fourOverThree - (9.0 * invZi - 4.0 * invZi3 + invZi5) / 6.0;
                up[3 * i] += Mxx * f[3 * i] * nf;
                up[3 * i + 1] += Mxx * f[3 * i + 1] * nf;
                up[3 * i + 2] += Mzz * f[3 * i + 2] * nf;
            }
            for (long j = i + 1; j < n; ++j) {
                double d0 = inva * (r[3 * i] - r[3 * j]);
                double d1 = inva * (r[3 * i + 1] - r[3 * j + 1]);
                double d2 = inva * (r[3 * i + 2] - r[3 * j + 2]);
                double rr = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                double r2 = rr * rr;
                double invr = 1.0 / rr;
                double invr2 = invr * invr;
                double Mxx, Mxy, Mxz, Myy, Myz, Mzz;
                if (rr > 2) {
                    double c1 = 1.0 + 2.0 / (3.0 * r2);
                    double c2 = (1.0 - 2.0 * invr2) * invr2;
                    Mxx = (c1 + c2 * d0 * d0) * invr;
                    Mxy = (c2 * d0 * d1) * invr;
                    Mxz = (c2 * d0 * d2) * invr;
                    Myy = (c1 + c2 * d1 * d1) * invr;
                    Myz = (c2 * d1 * d2) * invr;
                    Mzz = (c1 + c2 * d2 * d2) * invr;
                } else {
                    double c1 = fourOverThree * (1.0 - 0.28125 * rr);
                    double c2 = fourOverThree * 0.09375 * invr;
                    Mxx = c1 + c2 * d0 * d0;
                    Mxy = c2 * d0 * d1;
                    Mxz = c2 * d0 * d2;
                    Myy = c1 + c2 * d1 * d1;
                    Myz = c2 * d1 * d2;
                    Mzz = c1 + c2 * d2 * d2;
                }
                double Myx = Mxy, Mzx = Mxz, Mzy = Myz;
                d2 = (r[3 * i + 2] + r[3 * j + 2]) / a;
                double hj = r[3 * j + 2] / a;
                double h_hat = hj / d2;
                double invR = 1.0 / sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                double ex = d0 * invR, ey = d1 * invR, ez = d2 * invR;
                double ez2 = ez * ez;
                double invR3 = invR * invR * invR;
                double invR5 = invR3 * invR * invR;
                double t1 = (1.0 - h_hat) * ez2;
                double fact1 = -(3.0 * (1.0 + 2.0 * h_hat * t1) * invR + 2.0 * (1.0 - 3.0 * ez2) * invR3 - 2.0 * (1.0 - 5.0 * ez2) * invR5) / 3.0;
                double fact2 = -(3.0 * (1.0 - 6.0 * h_hat * t1) * invR - 6.0 * (1.0 - 5.0 * ez2) * invR3 + 10.0 * (1.0 - 7.0 * ez2) * invR5) / 3.0;
                double fact3 = ez * (3.0 * h_hat * (1.0 - 6.0 * t1) * invR - 6.0 * (1.0 - 5.0 * ez2) * invR3 + 10.0 * (2.0 - 7.0 * ez2) * invR5) * 2.0 / 3.0;
                double fact4 = ez * (3.0 * h_hat * invR - 10.0 * invR5) * 2.0 / 3.0;
                double fact5 = -(3.0 * h_hat * h_hat * ez2 * invR + 3.0 * ez2 * invR3 + (2.0 - 15.0 * ez2) * invR5) * 4.0 / 3.0;
                Mxx += fact1 + fact2 * ex * ex;
                Mxy += fact2 * ex * ey;
                Mxz += fact2 * ex * ez + fact3 * ex;
                Myx += fact2 * ey * ex;
                Myy += fact1 + fact2 * ey * ey;
                Myz += fact2 * ey * ez + fact3 * ey;
                Mzx += fact2 * ez * ex + fact4 * ex;
                Mzy += fact2 * ez * ey + fact4 * ey;
                Mzz += fact1 + fact2 * ez2 + fact3 * ez + fact4 * ez + fact5;
                up[3 * i] += (Mxx * f[3 * j] + Mxy * f[3 * j + 1] + Mxz * f[3 * j + 2]) * nf;
                up[3 * i + 1] += (Myx * f[3 * j] + Myy * f[3 * j + 1] + Myz * f[3 * j + 2]) * nf;
                up[3 * i + 2] += (Mzx * f[3 * j] + Mzy * f[3 * j + 1] + Mzz * f[3 * j + 2]) * nf;
                up[3 * j] += (Mxx * f[3 * i] + Myx * f[3 * i + 1] + Mzx * f[3 * i + 2]) * nf;
                up[3 * j + 1] += (Mxy * f[3 * i] + Myy * f[3 * i + 1] + Mzy * f[3 * i + 2]) * nf;
                up[3 * j + 2] += (Mxz * f[3 * i] + Myz * f[3 * i + 1] + Mzz * f[3 * i + 2]) * nf;
            }
        }
#pragma omp critical
        {
            for (long k = 0; k < 3 * n; ++k) u[k] += up[k];
        }
        free(up);
    }
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
