/*
 * p122_oracle.c -- CPU restatement of ParaFEM's p122: 3-D strain of an
 * elastic-plastic (Mohr-Coulomb) solid by the viscoplastic strain method,
 * with element-by-element PCG solves (src/programs/5th_ed/p122/p122.f90),
 * for 20-node or 8-node bricks, under load control, displacement control
 * (fixed freedoms by the penalty method) or both.
 *
 * TEST INFRASTRUCTURE ONLY, like p121_oracle.c: only the test suite, the
 * smoke check and the CPU baseline leg of the benchmark load it.
 *
 * Layouts are p121's (see p121_oracle.c).  Stresses and strains use nst = 6
 * in the order x, y, z, xy, yz, zx; evpt and tensor are (6, nip, nels).
 * Compiled with -ffp-contract=off (Fortran evaluation order).
 *
 * Parity pin: the restatement reproduces the reference's recorded book run
 * (examples/5th_ed/p122/book/p122.res, 20-node bricks, load control) and
 * demo run (examples/5th_ed/p122/demo/p122_demo.res and its ensi.DISPL
 * files, 8-node bricks, 19 fixed freedoms) increment by increment.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_sample(int nip, double *s, double *wt, int exact_weights);   /* p121_oracle.c */
void orc_shape_der20(double *der, double xi, double eta, double zeta);
void orc_shape_der8(double *der, double xi, double eta, double zeta);   /* p123_oracle.c */
void orc_deemat(double *dee, double e, double v);
double orc_determinant(const double *j);
void orc_invert3(double *m);
void orc_beemat(double *bee, const double *deriv);
void orc_form_storkm(int nels, int nip, int exact_weights, const double *g_coord, const double *e_el,
                     const double *v_el, int per_element, double *storkm);

/* INVAR, nst = 6 (src/modules/shared/new_library.f90:1813-1916) */
void orc_invar(const double *s, double *sigm, double *dsbar, double *theta)
{
    double sq3 = sqrt(3.0);
    double s1 = s[0], s2 = s[1], s3 = s[2], s4 = s[3], s5 = s[4], s6 = s[5];
    *sigm = (s1 + s2 + s3) / 3.0;
    double d2 = ((s1 - s2) * (s1 - s2) + (s2 - s3) * (s2 - s3) + (s3 - s1) * (s3 - s1)) / 6.0 + s4 * s4 + s5 * s5 +
                s6 * s6;
    double ds1 = s1 - *sigm, ds2 = s2 - *sigm, ds3 = s3 - *sigm;
    double d3 = ds1 * ds2 * ds3 - ds1 * s5 * s5 - ds2 * s6 * s6 - ds3 * s4 * s4 + 2.0 * s4 * s5 * s6;
    *dsbar = sq3 * sqrt(d2);
    if (*dsbar < 1.e-10) {
        *theta = 0.0;
    } else {
        double r = sqrt(d2);
        double sine = -3.0 * sq3 * d3 / (2.0 * (r * r * r));
        if (sine > 1.0) sine = 1.0;
        if (sine < -1.0) sine = -1.0;
        *theta = asin(sine) / 3.0;
    }
}

/* MOCOUF (new_library.f90:2364-2417) */
double orc_mocouf(double phi, double c, double sigm, double dsbar, double theta)
{
    double phir = phi * 4.0 * atan(1.0) / 180.0;
    double snph = sin(phir), csph = cos(phir), csth = cos(theta), snth = sin(theta);
    return snph * sigm + dsbar * (csth / sqrt(3.0) - snth * snph / 3.0) - c * csph;
}

/* MOCOUQ (new_library.f90:2423-2490) */
void orc_mocouq(double psi, double dsbar, double theta, double *dq1, double *dq2, double *dq3)
{
    double psir = psi * 4.0 * atan(1.0) / 180.0;
    double snth = sin(theta), snps = sin(psir), sq3 = sqrt(3.0);
    *dq1 = snps;
    if (fabs(snth) > 0.49) {
        double c1 = 1.0;
        if (snth < 0.0) c1 = -1.0;
        *dq2 = (sq3 * 0.5 - c1 * snps * 0.5 / sq3) * sq3 * 0.5 / dsbar;
        *dq3 = 0.0;
    } else {
        double csth = cos(theta), cs3th = cos(3.0 * theta), tn3th = tan(3.0 * theta), tnth = snth / csth;
        *dq2 = sq3 * csth / dsbar * ((1.0 + tnth * tn3th) + snps * (tn3th - tnth) / sq3) * 0.5;
        *dq3 = 0.5 * 3.0 * (sq3 * snth + snps * csth) / (cs3th * dsbar * dsbar);
    }
}

/* FORMM, nst = 6 (new_library.f90:85-198).  m(6,6) column-major. */
void orc_formm(const double *stress, double *m1, double *m2, double *m3)
{
    double sx = stress[0], sy = stress[1], sz = stress[2], txy = stress[3], tyz = stress[4], tzx = stress[5];
    double sigm = (sx + sy + sz) / 3.0, dx = sx - sigm, dy = sy - sigm, dz = sz - sigm;
#define M(m, i, j) m[((i) - 1) + 6 * ((j) - 1)]
    memset(m1, 0, 36 * sizeof(double));
    memset(m2, 0, 36 * sizeof(double));
    memset(m3, 0, 36 * sizeof(double));
    for (int i = 1; i <= 3; ++i)
        for (int j = 1; j <= 3; ++j) M(m1, i, j) = 1.0 / (3.0 * sigm);
    for (int i = 1; i <= 3; ++i) {
        M(m2, i, i) = 2.0;
        M(m2, i + 3, i + 3) = 6.0;
    }
    M(m2, 1, 2) = -1.0; M(m2, 1, 3) = -1.0; M(m2, 2, 3) = -1.0;
    M(m3, 1, 1) = dx; M(m3, 1, 2) = dz; M(m3, 1, 3) = dy; M(m3, 1, 4) = txy; M(m3, 1, 5) = -2.0 * tyz;
    M(m3, 1, 6) = tzx; M(m3, 2, 2) = dy; M(m3, 2, 3) = dx; M(m3, 2, 4) = txy; M(m3, 2, 5) = tyz;
    M(m3, 2, 6) = -2.0 * tzx; M(m3, 3, 3) = dz; M(m3, 3, 4) = -2.0 * txy; M(m3, 3, 5) = tyz; M(m3, 3, 6) = tzx;
    M(m3, 4, 4) = -3.0 * dz; M(m3, 4, 5) = 3.0 * tzx; M(m3, 4, 6) = 3.0 * tyz; M(m3, 5, 5) = -3.0 * dx;
    M(m3, 5, 6) = 3.0 * txy; M(m3, 6, 6) = -3.0 * dy;
    for (int i = 1; i <= 6; ++i)
        for (int j = i + 1; j <= 6; ++j) {
            M(m1, j, i) = M(m1, i, j);
            M(m2, j, i) = M(m2, i, j);
            M(m3, j, i) = M(m3, i, j);
        }
    for (int k = 0; k < 36; ++k) {
        m1[k] = m1[k] / 3.0;
        m2[k] = m2[k] / 3.0;
        m3[k] = m3[k] / 3.0;
    }
#undef M
}

/* u(g) += utemp: serial SCATTER, equation 0 is the dummy slot; nt freedoms
 * per element */
static void scatter_nt(int nels, int nt, const int *g_g, const double *ut, double *u0)
{
    for (int e = 0; e < nels; ++e)
        for (int i = 0; i < nt; ++i) u0[g_g[(size_t)nt * e + i]] += ut[(size_t)nt * e + i];
}

/* utemp(:,e) = storkm(:,:,e) . v(g(:,e)) for every element */
static void products(int nels, int nt, const int *g_g, const double *km, const double *v0, double *ut)
{
#pragma omp parallel for schedule(static)
    for (int e = 0; e < nels; ++e) {
        const double *k = &km[(size_t)nt * nt * e];
        double pe[60], acc[60];
        for (int i = 0; i < nt; ++i) { pe[i] = v0[g_g[(size_t)nt * e + i]]; acc[i] = 0.0; }
        for (int j = 0; j < nt; ++j)
            for (int i = 0; i < nt; ++i) acc[i] = acc[i] + k[i + nt * j] * pe[j];
        memcpy(&ut[(size_t)nt * e], acc, sizeof(double) * nt);
    }
}

/* SHAPE_DER of the element's nod-node brick */
static void shape_der(int nod, double *der, double xi, double eta, double zeta)
{
    if (nod == 8) orc_shape_der8(der, xi, eta, zeta);
    else orc_shape_der20(der, xi, eta, zeta);
}

/* BEEMAT for nod nodes (src/modules/shared/new_library.f90): bee(6, 3 nod) */
static void beemat_n(int nod, double *bee, const double *deriv)
{
    memset(bee, 0, sizeof(double) * 18 * nod);
#define B(r, c) bee[((r) - 1) + 6 * ((c) - 1)]
    for (int m = 1; m <= nod; ++m) {
        int n = 3 * m, k = n - 1, l = k - 1;
        double x = deriv[0 + 3 * (m - 1)], y = deriv[1 + 3 * (m - 1)], z = deriv[2 + 3 * (m - 1)];
        B(1, l) = x; B(4, k) = x; B(6, n) = x;
        B(2, k) = y; B(4, l) = y; B(5, n) = y;
        B(3, n) = z; B(5, k) = z; B(6, l) = z;
    }
#undef B
}

/* storkm of 8-node bricks, one material (p122.f90:76-84): the sum over the
 * Gauss points of MATMUL(MATMUL(TRANSPOSE(bee), dee), bee) * det * w */
static void form_storkm8(int nels, int nip, const double *g_coord, double e, double v, double *storkm)
{
    double *pts = (double *)malloc(sizeof(double) * nip * 3), *wts = (double *)malloc(sizeof(double) * nip);
    orc_sample(nip, pts, wts, 0);
    double dee[36];
    orc_deemat(dee, e, v);
#pragma omp parallel for schedule(static)
    for (int el = 0; el < nels; ++el) {
        double der[24], jac[9], deriv[24], bee[144], btd[144];
        double *km = &storkm[(size_t)576 * el];
        const double *co = &g_coord[(size_t)24 * el];
        memset(km, 0, 576 * sizeof(double));
        for (int i = 0; i < nip; ++i) {
            orc_shape_der8(der, pts[i], pts[i + nip], pts[i + 2 * nip]);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double s = 0.0;
                    for (int k = 0; k < 8; ++k) s += der[a + 3 * k] * co[k + 8 * b];
                    jac[a + 3 * b] = s;
                }
            double det = orc_determinant(jac);
            orc_invert3(jac);
            for (int l = 0; l < 8; ++l)
                for (int a = 0; a < 3; ++a) {
                    double s = 0.0;
                    for (int k = 0; k < 3; ++k) s += jac[a + 3 * k] * der[k + 3 * l];
                    deriv[a + 3 * l] = s;
                }
            beemat_n(8, bee, deriv);
            for (int r = 0; r < 24; ++r)
                for (int c = 0; c < 6; ++c) {
                    double s = 0.0;
                    for (int k = 0; k < 6; ++k) s += bee[k + 6 * r] * dee[k + 6 * c];
                    btd[r + 24 * c] = s;
                }
            for (int c = 0; c < 24; ++c)
                for (int r = 0; r < 24; ++r) {
                    double s = 0.0;
                    for (int k = 0; k < 6; ++k) s += btd[r + 24 * k] * bee[k + 6 * c];
                    km[r + 24 * c] = km[r + 24 * c] + s * det * wts[i];
                }
        }
    }
    free(pts);
    free(wts);
}

/* form_storkm8 for the tests: g_coord(8,3,nels) -> storkm(24,24,nels) */
void orc_form_storkm8(int nels, int nip, const double *g_coord, double e, double v, double *storkm)
{
    form_storkm8(nels, nip, g_coord, e, v, storkm);
}

/* checon_par (src/modules/mpi/maths.f90:999-1069): converged when
 * max|xnew - x| / max|xnew| <= tol; then x = xnew.  Vectors are 1-based. */
static int checon(int neq, const double *xnew, double tol, double *x)
{
    double maxl = 0.0, maxd = 0.0;
    for (int q = 1; q <= neq; ++q) {
        double a = fabs(xnew[q]);
        if (a > maxl) maxl = a;
        double b = fabs(xnew[q] - x[q]);
        if (b > maxd) maxd = b;
    }
    for (int q = 1; q <= neq; ++q) x[q] = xnew[q];
    return maxd / maxl <= tol;
}

/* The p122 solve (p122.f90:78-225) for nod-node bricks (8 or 20).
 * ld0: the assembled nodal loads (neq), or NULL when no node is loaded.
 * Fixed freedoms (p122.f90:96-113, 122-139, 153-158): equations fix_eq[i]
 * (1-based) with prescribed values fix_val[i]; the penalty 1e20 is added to
 * their diagonal and store = the penalised diagonal.  On the first plastic
 * iteration of an increment loads(fix) = store * val * qinc and the product
 * at those equations is p * store; after it loads(fix) = 0 and the product is
 * 0 there.  Loaded nodes, when present, replace the whole load vector on the
 * first plastic iteration (loads = ld0 qinc + bdylds), as the reference does.
 * out[6*iy + k] for each increment: totd(1), tensor(3,1,1), tensor(1,1,1),
 * tensor(2,1,1), cj iterations, plastic iterations.  totd_out (neq x incs,
 * may be NULL) receives the total displacements after each increment.
 * Returns the increments run. */
int orc_p122n(int nod, int nels, int neq, const int *g_g, const double *g_coord, int nip, double phi, double c,
              double psi, double e, double v, int incs, const double *qinc, int plasits, int cjits, double plastol,
              double cjtol, const double *ld0, int nfix, const int *fix_eq, const double *fix_val, double *out,
              double *totd_out)
{
    const int nt = 3 * nod, nb = 6 * nt;
    const double penalty = 1.e20;
    size_t n1 = (size_t)neq + 1;
    double *km = (double *)malloc(sizeof(double) * nt * nt * (size_t)nels);
    if (nod == 8) {
        form_storkm8(nels, nip, g_coord, e, v, km);
    } else {
        double ev[1] = {e}, vv[1] = {v};
        orc_form_storkm(nels, nip, 0, g_coord, ev, vv, 0, km);
    }
    /* B and det*w at every Gauss point (the reference recomputes the same values) */
    double *bee = (double *)malloc(sizeof(double) * nb * (size_t)nip * nels);
    double *detw = (double *)malloc(sizeof(double) * (size_t)nip * nels);
    double *dets = (double *)malloc(sizeof(double) * (size_t)nip * nels);
    double *pts = (double *)malloc(sizeof(double) * 3 * nip), *wts = (double *)malloc(sizeof(double) * nip);
    orc_sample(nip, pts, wts, 0);
#pragma omp parallel for schedule(static)
    for (int el = 0; el < nels; ++el) {
        double der[60], jac[9], deriv[60];
        const double *co = &g_coord[(size_t)nt * el];
        for (int i = 0; i < nip; ++i) {
            shape_der(nod, der, pts[i], pts[i + nip], pts[i + 2 * nip]);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double s = 0.0;
                    for (int k = 0; k < nod; ++k) s += der[a + 3 * k] * co[k + nod * b];
                    jac[a + 3 * b] = s;
                }
            double det = orc_determinant(jac);
            orc_invert3(jac);
            for (int l = 0; l < nod; ++l)
                for (int a = 0; a < 3; ++a) {
                    double s = 0.0;
                    for (int k = 0; k < 3; ++k) s += jac[a + 3 * k] * der[k + 3 * l];
                    deriv[a + 3 * l] = s;
                }
            beemat_n(nod, &bee[nb * ((size_t)el * nip + i)], deriv);
            dets[(size_t)el * nip + i] = det;
            detw[(size_t)el * nip + i] = wts[i];
        }
    }
    double dee[36];
    orc_deemat(dee, e, v);
    double *diag = (double *)calloc(n1, sizeof(double));
    for (int el = 0; el < nels; ++el)
        for (int i = 0; i < nt; ++i) diag[g_g[(size_t)nt * el + i]] += km[(size_t)nt * nt * el + (nt + 1) * i];
    double *store = (double *)calloc(nfix > 0 ? nfix : 1, sizeof(double));
    for (int i = 0; i < nfix; ++i) {
        diag[fix_eq[i]] = diag[fix_eq[i]] + penalty;
        store[i] = diag[fix_eq[i]];
    }
    double *dinv = (double *)calloc(n1, sizeof(double));
    for (size_t q = 1; q < n1; ++q) dinv[q] = 1.0 / diag[q];
    double pi = acos(-1.0), snph = sin(phi * pi / 180.0);
    double dt = 4.0 * (1.0 + v) * (1.0 - 2.0 * v) / (e * (1.0 - 2.0 * v + snph * snph));
    size_t ngp = (size_t)nip * nels;
    double *evpt = (double *)calloc(6 * ngp, sizeof(double)), *tensor = (double *)calloc(6 * ngp, sizeof(double));
    double *loads = (double *)calloc(n1, sizeof(double)), *bdylds = (double *)calloc(n1, sizeof(double));
    double *oldis = (double *)calloc(n1, sizeof(double)), *totd = (double *)calloc(n1, sizeof(double));
    double *r = (double *)calloc(n1, sizeof(double)), *p = (double *)calloc(n1, sizeof(double));
    double *x = (double *)calloc(n1, sizeof(double)), *xnew = (double *)calloc(n1, sizeof(double));
    double *u = (double *)calloc(n1, sizeof(double)), *d = (double *)calloc(n1, sizeof(double));
    double *ut = (double *)malloc(sizeof(double) * nt * (size_t)nels);
    int iy = 0;
    for (iy = 1; iy <= incs; ++iy) {
        int plasiters = 0, cjtot = 0, plastic_converged = 0;
        memset(bdylds, 0, n1 * sizeof(double));
        memset(evpt, 0, 6 * ngp * sizeof(double));
        for (;;) {
            ++plasiters;
            memset(loads, 0, n1 * sizeof(double));
            if (plasiters == 1) {
                for (int i = 0; i < nfix; ++i) loads[fix_eq[i]] = store[i] * fix_val[i] * qinc[iy - 1];
                if (ld0) {
                    for (size_t q = 1; q < n1; ++q) loads[q] = ld0[q - 1] * qinc[iy - 1];
                    for (size_t q = 1; q < n1; ++q) loads[q] = loads[q] + bdylds[q];
                }
            } else {
                if (ld0)
                    for (size_t q = 1; q < n1; ++q) loads[q] = ld0[q - 1] * qinc[iy - 1];
                for (size_t q = 1; q < n1; ++q) loads[q] = loads[q] + bdylds[q];
                for (int i = 0; i < nfix; ++i) loads[fix_eq[i]] = 0.0;
            }
            /* r = loads - K x, d = M^-1 r, p = d */
            x[0] = 0.0;
            products(nels, nt, g_g, km, x, ut);
            memset(r, 0, n1 * sizeof(double));
            scatter_nt(nels, nt, g_g, ut, r);
            for (size_t q = 1; q < n1; ++q) r[q] = loads[q] - r[q];
            for (size_t q = 1; q < n1; ++q) { d[q] = dinv[q] * r[q]; p[q] = d[q]; }
            int cjiters = 0;
            for (;;) {
                ++cjiters;
                p[0] = 0.0;
                products(nels, nt, g_g, km, p, ut);
                memset(u, 0, n1 * sizeof(double));
                scatter_nt(nels, nt, g_g, ut, u);
                for (int i = 0; i < nfix; ++i) u[fix_eq[i]] = plasiters == 1 ? p[fix_eq[i]] * store[i] : 0.0;
                double up = 0.0, pu = 0.0;
                for (size_t q = 1; q < n1; ++q) up += r[q] * d[q];
                for (size_t q = 1; q < n1; ++q) pu += p[q] * u[q];
                double alpha = up / pu;
                for (size_t q = 1; q < n1; ++q) xnew[q] = x[q] + p[q] * alpha;
                for (size_t q = 1; q < n1; ++q) r[q] = r[q] - u[q] * alpha;
                for (size_t q = 1; q < n1; ++q) d[q] = dinv[q] * r[q];
                double rd = 0.0;
                for (size_t q = 1; q < n1; ++q) rd += r[q] * d[q];
                double beta = rd / up;
                for (size_t q = 1; q < n1; ++q) p[q] = d[q] + p[q] * beta;
                int conv = checon(neq, xnew, cjtol, x);
                if (conv || cjiters == cjits) break;
            }
            cjtot += cjiters;
            for (size_t q = 1; q < n1; ++q) loads[q] = xnew[q];
            plastic_converged = checon(neq, loads, plastol, oldis);
            if (plasiters == 1) plastic_converged = 0;
            int last = plastic_converged || plasiters == plasits;
            if (last) memset(bdylds, 0, n1 * sizeof(double));
            loads[0] = 0.0;
            /* stresses, yield, viscoplastic strains and body loads (p122.f90:172-202) */
#pragma omp parallel for schedule(static)
            for (int el = 0; el < nels; ++el) {
                double eld[60], bload[60], eps[6], sigma[6], stress[6], devp[6], evp[6], erate[6];
                double m1[36], m2[36], m3[36], flow[36];
                for (int k = 0; k < nt; ++k) { eld[k] = loads[g_g[(size_t)nt * el + k]]; bload[k] = 0.0; }
                for (int i = 0; i < nip; ++i) {
                    size_t gi = (size_t)el * nip + i;
                    const double *b = &bee[nb * gi];
                    double *ev = &evpt[6 * gi], *tn = &tensor[6 * gi];
                    for (int a = 0; a < 6; ++a) {
                        double s = 0.0;
                        for (int k = 0; k < nt; ++k) s += b[a + 6 * k] * eld[k];
                        eps[a] = s;
                    }
                    for (int a = 0; a < 6; ++a) eps[a] = eps[a] - ev[a];
                    for (int a = 0; a < 6; ++a) {
                        double s = 0.0;
                        for (int k = 0; k < 6; ++k) s += dee[a + 6 * k] * eps[k];
                        sigma[a] = s;
                    }
                    for (int a = 0; a < 6; ++a) stress[a] = sigma[a] + tn[a];
                    double sigm, dsbar, theta;
                    orc_invar(stress, &sigm, &dsbar, &theta);
                    double f = orc_mocouf(phi, c, sigm, dsbar, theta);
                    if (last) {
                        for (int a = 0; a < 6; ++a) devp[a] = stress[a];
                    } else if (f >= 0.0) {
                        double dq1, dq2, dq3;
                        orc_mocouq(psi, dsbar, theta, &dq1, &dq2, &dq3);
                        orc_formm(stress, m1, m2, m3);
                        for (int k = 0; k < 36; ++k) flow[k] = f * (m1[k] * dq1 + m2[k] * dq2 + m3[k] * dq3);
                        for (int a = 0; a < 6; ++a) {
                            double s = 0.0;
                            for (int k = 0; k < 6; ++k) s += flow[a + 6 * k] * stress[k];
                            erate[a] = s;
                        }
                        for (int a = 0; a < 6; ++a) evp[a] = erate[a] * dt;
                        for (int a = 0; a < 6; ++a) ev[a] = ev[a] + evp[a];
                        for (int a = 0; a < 6; ++a) {
                            double s = 0.0;
                            for (int k = 0; k < 6; ++k) s += dee[a + 6 * k] * evp[k];
                            devp[a] = s;
                        }
                    }
                    if (f >= 0.0) {
                        for (int k = 0; k < nt; ++k) {
                            double s = 0.0;
                            for (int a = 0; a < 6; ++a) s += b[a + 6 * k] * devp[a];
                            bload[k] = bload[k] + s * dets[gi] * detw[gi];
                        }
                    }
                    if (last)
                        for (int a = 0; a < 6; ++a) tn[a] = stress[a];
                }
                memcpy(&ut[(size_t)nt * el], bload, sizeof(double) * nt);
            }
            scatter_nt(nels, nt, g_g, ut, bdylds);
            bdylds[0] = 0.0;
            if (last) break;
        }
        for (size_t q = 1; q < n1; ++q) totd[q] = totd[q] + loads[q];
        double *o = &out[6 * (iy - 1)];
        o[0] = totd[1];
        o[1] = tensor[2];
        o[2] = tensor[0];
        o[3] = tensor[1];
        o[4] = cjtot;
        o[5] = plasiters;
        if (totd_out) memcpy(&totd_out[(size_t)neq * (iy - 1)], totd + 1, sizeof(double) * neq);
        if (plasiters == plasits) break;
    }
    int done = iy > incs ? incs : iy;
    free(km); free(bee); free(detw); free(dets); free(pts); free(wts); free(diag); free(dinv); free(store);
    free(evpt); free(tensor); free(loads); free(bdylds); free(oldis); free(totd); free(r); free(p); free(x);
    free(xnew); free(u); free(d); free(ut);
    return done;
}

/* 20-node bricks under load control (the book run's case) */
int orc_p122(int nels, int neq, const int *g_g, const double *g_coord, int nip, double phi, double c, double psi,
             double e, double v, int incs, const double *qinc, int plasits, int cjits, double plastol, double cjtol,
             const double *ld0, double *out, double *totd_out)
{
    return orc_p122n(20, nels, neq, g_g, g_coord, nip, phi, c, psi, e, v, incs, qinc, plasits, cjits, plastol, cjtol,
                     ld0, 0, NULL, NULL, out, totd_out);
}
