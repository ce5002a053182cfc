/* p121_cpu.c -- the timed CPU baseline of p121's solve (BENCH AND TEST
 * INFRASTRUCTURE ONLY; the product library never links or calls it).
 *
 * p121_oracle.c restates p121 in the Fortran's evaluation order for parity
 * (-ffp-contract=off, serial GATHER/SCATTER and dot products).  This file is
 * the same algorithm written for speed on the host's cores, the way
 * ParaFEM's MPI p121 spreads every loop of its iteration over the ranks:
 *   - src/programs/5th_ed/p121/p121.f90:54-64 (storkm), formed by node pairs
 *     (M_ab = sum det w g_a g_b', then the isotropic D's three terms), with
 *     the element loop over all threads;
 *   - p121.f90:90-104 (the PCG iteration): GATHER fused into the element
 *     products, the element products, SCATTER as a node-centric sum over an
 *     inverse-connectivity list (each equation sums its contributions in
 *     ascending element order, as the serial SCATTER does, so the result
 *     does not depend on the thread count), the dot products
 *     (maths.f90:168-215) as per-thread partials combined in thread order,
 *     the axpy updates and checon_par (maths.f90:999-1069), every loop
 *     split over all threads;
 *   - built at -O3 with floating-point contraction allowed.
 * The mesh is the fixed-base, top-pressure 20-node cube of GEOMETRY_20BXZ
 * (geometry.f90:172-290), numbered by REARRANGE + find_g3
 * (new_library.f90:3059-3212) through the routines of p121_oracle.c.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void orc_geometry_20bxz(int iel, int nxe, int nze, double aa, double bb, double cc, double *coord, int *num);
void orc_rearrange(int nr, int *rest);
void orc_find_g3(const int *num, int *g, int nr, const int *rest);
int orc_sample(int nip, double *s, double *wt, int exact_weights);
void orc_shape_der20(double *der, double xi, double eta, double zeta);
double orc_determinant(const double *j);
void orc_invert3(double *m);

typedef struct {
    int nels, neq, nthreads, iters;
    int *g_g;          /* [60*nels] 1-based equations, 0 = restrained */
    double *coord;     /* [60*nels] g_coord(20,3,e) */
    double *storkm;    /* [3600*nels] storkm(60,60,e) column-major */
    int *eptr, *elist; /* CSR equation q (1..neq) -> utemp positions 60e+i, ascending e */
    double *rhs, *dinv, *x, *r, *d, *p, *u, *utemp;
    double *part;      /* [8*nthreads] per-thread partials */
    double up, ff, metric;
} Cpu121;

static int nthreads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int thread_id(void)
{
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

/* The cube of 20-node bricks, every dof of the base face (z = -nze) fixed,
 * uniform pressure on the top face (z = 0) with total load -1 as consistent
 * nodal forces: +p/12 at each face corner, -p/3 at each mid-side node. */
static int build_cube(Cpu121 *h, int nxe, int nye, int nze)
{
    const int nels = nxe * nye * nze;
    int *g_num = (int *)malloc(sizeof(int) * 20 * (size_t)nels);
    h->coord = (double *)malloc(sizeof(double) * 60 * (size_t)nels);
    h->g_g = (int *)malloc(sizeof(int) * 60 * (size_t)nels);
    if (!g_num || !h->coord || !h->g_g) { free(g_num); return -1; }
    int nn = 0;
#pragma omp parallel for schedule(static) reduction(max : nn)
    for (int e = 0; e < nels; ++e) {
        orc_geometry_20bxz(e + 1, nxe, nze, 1.0, 1.0, 1.0, h->coord + 60 * (size_t)e, g_num + 20 * (size_t)e);
        for (int a = 0; a < 20; ++a) if (g_num[20 * (size_t)e + a] > nn) nn = g_num[20 * (size_t)e + a];
    }
    char *base = (char *)calloc((size_t)nn + 1, 1);
    static const int base_local[8] = {0, 6, 7, 8, 11, 12, 18, 19};   /* z = zb nodes */
    for (int e = 0; e < nels; ++e)
        if (e % (nxe * nze) >= nxe * (nze - 1))
            for (int k = 0; k < 8; ++k) base[g_num[20 * (size_t)e + base_local[k]]] = 1;
    int nr = 1;
    for (int n = 1; n <= nn; ++n) nr += base[n];
    int *rest = (int *)malloc(sizeof(int) * 4 * (size_t)nr);
    rest[0] = rest[1] = rest[2] = rest[3] = 1;          /* a free first row keeps find_g3 inside rest */
    for (int n = 1, k = 1; n <= nn; ++n)
        if (base[n]) { rest[4 * k] = n; rest[4 * k + 1] = rest[4 * k + 2] = rest[4 * k + 3] = 0; ++k; }
    orc_rearrange(nr, rest);
    int neq = 0;
#pragma omp parallel for schedule(static) reduction(max : neq)
    for (int e = 0; e < nels; ++e) {
        int *g = h->g_g + 60 * (size_t)e;
        orc_find_g3(g_num + 20 * (size_t)e, g, nr, rest);
        for (int i = 0; i < 60; ++i) if (g[i] > neq) neq = g[i];
    }
    h->nels = nels;
    h->neq = neq;
    h->rhs = (double *)calloc((size_t)neq + 1, sizeof(double));
    const double pr = 1.0 / ((double)nxe * nye);
    for (int e = 0; e < nels; ++e)
        if (e % (nxe * nze) < nxe) {
            static const int corner[4] = {3, 5, 15, 17}, mid[4] = {4, 10, 11, 16};
            for (int k = 0; k < 4; ++k) h->rhs[h->g_g[60 * (size_t)e + 3 * corner[k] - 1]] += pr / 12.0;
            for (int k = 0; k < 4; ++k) h->rhs[h->g_g[60 * (size_t)e + 3 * mid[k] - 1]] -= pr / 3.0;
        }
    h->rhs[0] = 0.0;
    free(base);
    free(rest);
    free(g_num);
    return 0;
}

/* storkm by node pairs: M_ab = sum over the Gauss points of det*w*g_a g_b'
 * (g = J^-1 dN), then K(3a+i, 3b+j) = lam M_ab(i,j) + mu M_ab(j,i)
 * + mu delta_ij trace(M_ab), which is B'DB of DEEMAT's isotropic D
 * (new_library.f90:1671-1689) with BEEMAT's zeros skipped. */
static void form_storkm(Cpu121 *h, int nip, double E, double nu)
{
    double pts[27 * 3], wts[27], der[27][60];
    orc_sample(nip, pts, wts, 0);
    for (int g = 0; g < nip; ++g) orc_shape_der20(der[g], pts[g], pts[g + nip], pts[g + 2 * nip]);
    const double vv = (1.0 - 2.0 * nu) / (1.0 - nu) * 0.5;
    const double den = 2.0 * (1.0 + nu) * vv;
    const double lam = nu / (1.0 - nu) * E / den, mu = vv * E / den;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < h->nels; ++e) {
        const double *co = h->coord + 60 * (size_t)e;
        double M[210][9];
        memset(M, 0, sizeof M);
        for (int g = 0; g < nip; ++g) {
            double jac[9];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double s = 0.0;
                    for (int k = 0; k < 20; ++k) s += der[g][a + 3 * k] * co[k + 20 * b];
                    jac[a + 3 * b] = s;
                }
            const double dw = orc_determinant(jac) * wts[g];
            orc_invert3(jac);
            double gr[20][3];
            for (int l = 0; l < 20; ++l)
                for (int a = 0; a < 3; ++a)
                    gr[l][a] = jac[a] * der[g][3 * l] + jac[a + 3] * der[g][3 * l + 1] + jac[a + 6] * der[g][3 * l + 2];
            int pq = 0;
            for (int a = 0; a < 20; ++a) {
                const double s0 = dw * gr[a][0], s1 = dw * gr[a][1], s2 = dw * gr[a][2];
                for (int b = a; b < 20; ++b, ++pq) {
                    double *m = M[pq];
                    m[0] += s0 * gr[b][0]; m[1] += s0 * gr[b][1]; m[2] += s0 * gr[b][2];
                    m[3] += s1 * gr[b][0]; m[4] += s1 * gr[b][1]; m[5] += s1 * gr[b][2];
                    m[6] += s2 * gr[b][0]; m[7] += s2 * gr[b][1]; m[8] += s2 * gr[b][2];
                }
            }
        }
        double *km = h->storkm + 3600 * (size_t)e;
        int pq = 0;
        for (int a = 0; a < 20; ++a)
            for (int b = a; b < 20; ++b, ++pq) {
                const double *m = M[pq];
                const double tr = m[0] + m[4] + m[8];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        const double v = lam * m[3 * i + j] + mu * m[3 * j + i] + (i == j ? mu * tr : 0.0);
                        km[(3 * a + i) + 60 * (3 * b + j)] = v;
                        km[(3 * b + j) + 60 * (3 * a + i)] = v;
                    }
            }
    }
}

/* Inverse connectivity: for each equation the utemp positions 60e+i that
 * SCATTER adds into it, ascending in e (the serial SCATTER's order). */
static int build_csr(Cpu121 *h)
{
    const size_t nc = 60 * (size_t)h->nels;
    h->eptr = (int *)calloc((size_t)h->neq + 2, sizeof(int));
    h->elist = (int *)malloc(sizeof(int) * nc);
    if (!h->eptr || !h->elist) return -1;
    for (size_t k = 0; k < nc; ++k) h->eptr[h->g_g[k] + 1]++;
    for (int q = 1; q <= h->neq + 1; ++q) h->eptr[q] += h->eptr[q - 1];
    int *fill = (int *)malloc(sizeof(int) * ((size_t)h->neq + 1));
    memcpy(fill, h->eptr, sizeof(int) * ((size_t)h->neq + 1));
    for (size_t k = 0; k < nc; ++k) {
        const int q = h->g_g[k];
        if (q > 0) h->elist[fill[q]++] = (int)k;
    }
    free(fill);
    return 0;
}

/* Sums the per-thread partials of slot k in thread order. */
static double combine(const Cpu121 *h, int k, int is_max)
{
    double s = 0.0;
    for (int t = 0; t < h->nthreads; ++t) {
        const double v = h->part[8 * t + k];
        s = is_max ? (v > s ? v : s) : s + v;
    }
    return s;
}

void cpu121_destroy(void *ptr)
{
    Cpu121 *h = (Cpu121 *)ptr;
    if (!h) return;
    free(h->g_g); free(h->coord); free(h->storkm); free(h->eptr); free(h->elist);
    free(h->rhs); free(h->dinv); free(h->x); free(h->r); free(h->d); free(h->p); free(h->u);
    free(h->utemp); free(h->part);
    free(h);
}

/* Builds the cube, forms storkm (nip 8 or 27) with E and nu, the Jacobi
 * diagonal (p121.f90:65-69,86) and the scatter list.  NULL on failure. */
void *cpu121_create(int nxe, int nye, int nze, int nip, double E, double nu)
{
    Cpu121 *h = (Cpu121 *)calloc(1, sizeof(Cpu121));
    if (!h || build_cube(h, nxe, nye, nze) != 0) { cpu121_destroy(h); return NULL; }
    const size_t n1 = (size_t)h->neq + 1;
    h->storkm = (double *)malloc(sizeof(double) * 3600 * (size_t)h->nels);
    h->utemp = (double *)malloc(sizeof(double) * 60 * (size_t)h->nels);
    h->dinv = (double *)calloc(n1, sizeof(double));
    h->x = (double *)calloc(n1, sizeof(double));
    h->r = (double *)calloc(n1, sizeof(double));
    h->d = (double *)calloc(n1, sizeof(double));
    h->p = (double *)calloc(n1, sizeof(double));
    h->u = (double *)calloc(n1, sizeof(double));
    h->nthreads = nthreads();
    h->part = (double *)calloc(8 * (size_t)h->nthreads, sizeof(double));
    if (!h->storkm || !h->utemp || !h->dinv || !h->x || !h->r || !h->d || !h->p || !h->u || !h->part ||
        build_csr(h) != 0) {
        cpu121_destroy(h);
        return NULL;
    }
    form_storkm(h, nip, E, nu);
    free(h->coord);
    h->coord = NULL;
#pragma omp parallel for schedule(static)
    for (int q = 1; q <= h->neq; ++q) {
        double s = 0.0;
        for (int k = h->eptr[q]; k < h->eptr[q + 1]; ++k) {
            const size_t c = (size_t)h->elist[k];
            s += h->storkm[3600 * (c / 60) + 61 * (c % 60)];
        }
        h->dinv[q] = 1.0 / s;
    }
    return h;
}

int cpu121_neq(void *ptr) { return ((Cpu121 *)ptr)->neq; }
int cpu121_threads(void *ptr) { return ((Cpu121 *)ptr)->nthreads; }
double cpu121_metric(void *ptr) { return ((Cpu121 *)ptr)->metric; }

/* Copies storkm of elements [e0, e0+count) (column-major 60x60 each). */
void cpu121_get_storkm(void *ptr, int e0, int count, double *out)
{
    const Cpu121 *h = (const Cpu121 *)ptr;
    memcpy(out, h->storkm + 3600 * (size_t)e0, sizeof(double) * 3600 * (size_t)count);
}

/* g_g (60 x nels, 1-based) and the load vector (neq). */
void cpu121_get_problem(void *ptr, int *g_g, double *rhs)
{
    const Cpu121 *h = (const Cpu121 *)ptr;
    if (g_g) memcpy(g_g, h->g_g, sizeof(int) * 60 * (size_t)h->nels);
    if (rhs) memcpy(rhs, h->rhs + 1, sizeof(double) * h->neq);
}

/* PCG start (p121.f90:86-88): x = 0, r = f, d = diag^-1 r, p = d, up = r.d. */
void cpu121_init(void *ptr)
{
    Cpu121 *h = (Cpu121 *)ptr;
#pragma omp parallel
    {
        double rd = 0.0, ff = 0.0;
#pragma omp for schedule(static)
        for (int q = 1; q <= h->neq; ++q) {
            const double rv = h->rhs[q], dv = h->dinv[q] * rv;
            h->x[q] = 0.0;
            h->r[q] = rv;
            h->d[q] = dv;
            h->p[q] = dv;
            rd += rv * dv;
            ff += rv * rv;
        }
        h->part[8 * thread_id()] = rd;
        h->part[8 * thread_id() + 1] = ff;
    }
    h->up = combine(h, 0, 0);
    h->ff = combine(h, 1, 0);
    h->iters = 0;
    h->metric = 0.0;
}

/* Up to k PCG iterations of p121.f90:90-104 from the current state; stops
 * early when the test is met (stop_mode 0: checon_par's
 * max|xnew-x|/max|xnew| <= tol; 1: ||r||/||f|| <= tol; tol 0 never stops).
 * Returns the iterations run. */
int cpu121_iterate(void *ptr, int k, double tol, int stop_mode)
{
    Cpu121 *h = (Cpu121 *)ptr;
    const int nels = h->nels, neq = h->neq;
    int done = 0;
    h->p[0] = 0.0;
    for (; done < k; ++done) {
#pragma omp parallel
        {
            const int t = thread_id();
            /* GATHER + element products utemp(:,e) = storkm(:,:,e) pmul(:,e) */
#pragma omp for schedule(static)
            for (int e = 0; e < nels; ++e) {
                const int *g = h->g_g + 60 * (size_t)e;
                const double *km = h->storkm + 3600 * (size_t)e;
                double pe[60], acc[60];
                for (int i = 0; i < 60; ++i) { pe[i] = h->p[g[i]]; acc[i] = 0.0; }
                for (int j = 0; j < 60; ++j) {
                    const double pj = pe[j];
                    const double *col = km + 60 * j;
                    for (int i = 0; i < 60; ++i) acc[i] += col[i] * pj;
                }
                memcpy(h->utemp + 60 * (size_t)e, acc, sizeof acc);
            }
            /* SCATTER by equation, and p.u */
            double pu = 0.0;
#pragma omp for schedule(static)
            for (int q = 1; q <= neq; ++q) {
                double s = 0.0;
                for (int c = h->eptr[q]; c < h->eptr[q + 1]; ++c) s += h->utemp[h->elist[c]];
                h->u[q] = s;
                pu += h->p[q] * s;
            }
            h->part[8 * t] = pu;
#pragma omp barrier
            const double a = h->up / combine(h, 0, 0);
            /* xnew = x + alpha p, r -= alpha u, d = diag^-1 r; r.d, r.r and checon_par's maxima */
            double rd = 0.0, rr = 0.0, mx = 0.0, md = 0.0;
#pragma omp for schedule(static)
            for (int q = 1; q <= neq; ++q) {
                const double xo = h->x[q], xn = xo + h->p[q] * a;
                h->x[q] = xn;
                const double ax = fabs(xn), dx = fabs(xn - xo);
                mx = ax > mx ? ax : mx;
                md = dx > md ? dx : md;
                const double rn = h->r[q] - h->u[q] * a;
                h->r[q] = rn;
                const double dn = h->dinv[q] * rn;
                h->d[q] = dn;
                rd += rn * dn;
                rr += rn * rn;
            }
            h->part[8 * t + 1] = rd;
            h->part[8 * t + 2] = rr;
            h->part[8 * t + 3] = mx;
            h->part[8 * t + 4] = md;
#pragma omp barrier
            const double b = combine(h, 1, 0) / h->up;
#pragma omp for schedule(static)
            for (int q = 1; q <= neq; ++q) h->p[q] = h->d[q] + h->p[q] * b;
        }
        const double rd = combine(h, 1, 0), rr = combine(h, 2, 0);
        const double mx = combine(h, 3, 1), md = combine(h, 4, 1);
        h->up = rd;
        h->iters++;
        h->metric = stop_mode == 0 ? md / mx : sqrt(rr) / sqrt(h->ff);
        if (tol > 0.0 && h->metric <= tol) { ++done; break; }
    }
    return done;
}

/* The current iterate x (neq). */
void cpu121_get_x(void *ptr, double *x)
{
    const Cpu121 *h = (const Cpu121 *)ptr;
    memcpy(x, h->x + 1, sizeof(double) * h->neq);
}
