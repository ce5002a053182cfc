// pf_plastic.cu -- p122: 3-D strain of an elastic-plastic (Mohr-Coulomb)
// solid by the viscoplastic strain method (src/programs/5th_ed/p122/p122.f90),
// 20-node bricks or 8-node bricks, load control, displacement control (fixed
// freedoms by the penalty method) or both, on the GPU.
//
// Every plastic iteration is one warm-started element-by-element PCG solve
// (the p121 kernels: r = loads - K x, then p121's iteration with checon_par)
// followed by one pass over the Gauss points:
//   k_p122_bee       B (6 x 3 nod), det and weight at every Gauss point, once;
//   k_p122_plastic   one warp per element: eps = B u_e - evpt, sigma = D eps,
//                    stress = sigma + tensor; INVAR, MOCOUF; at a yielding
//                    point MOCOUQ, FORMM, the viscoplastic strain rate, evpt
//                    and the body loads B' D evp det w (p122.f90:172-202),
//                    summed over the Gauss points in order;
// and the body loads are added into bdylds by the node-centric scatter.
#include "pf_device.cuh"
#include "pfgpu.h"

#include <cmath>
#include <vector>

namespace pf {

namespace {

struct P122 {
    int nip = 0;
    double *bee = nullptr;     // [nels][nip][6 * 3 nod] column-major B
    double *detw = nullptr;    // [nels][nip][2]: det, weight
    double *evpt = nullptr;    // [nels][nip][6]
    double *tensor = nullptr;  // [nels][nip][6]
    double *ld0 = nullptr, *loads = nullptr, *bdylds = nullptr, *oldis = nullptr, *totd = nullptr;   // slots
    double *red = nullptr;     // [2 * G + 8] checon partials and results
    int *fslot = nullptr;      // [nfix] slots of the fixed freedoms
    double *fval = nullptr;    // [nfix] their prescribed values
};

void p122_free(P122 &q)
{
    double *ptrs[] = {q.bee, q.detw, q.evpt, q.tensor, q.ld0, q.loads, q.bdylds, q.oldis, q.totd, q.red, q.fval};
    for (double *x : ptrs)
        if (x) cudaFree(x);
    if (q.fslot) cudaFree(q.fslot);
    q = P122();
}

}  // namespace

// B, det and weight at Gauss point g of element e (thread per point), NOD-node bricks
template <int NOD>
__global__ void k_p122_bee(int nels, int nip, const double *__restrict__ gp, const double *__restrict__ coord,
                           double *__restrict__ bee, double *__restrict__ detw)
{
    constexpr int NE = 3 * NOD;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)nels * nip;
         t += (long long)gridDim.x * blockDim.x) {
        const size_t e = (size_t)(t / nip);
        const int g = (int)(t % nip);
        const double *co = coord + e * NE;
        double der[NE], jac[9];
        for (int l = 0; l < NOD; ++l) {
            if constexpr (NOD == 20) shape_der20(l, gp[4 * g], gp[4 * g + 1], gp[4 * g + 2], &der[3 * l]);
            else shape_der8(l, gp[4 * g], gp[4 * g + 1], gp[4 * g + 2], &der[3 * l]);
        }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                for (int k = 0; k < NOD; ++k) s += der[a + 3 * k] * co[k + NOD * b];
                jac[a + 3 * b] = s;
            }
        const double det = det_invert3(jac);
        double *B = bee + (size_t)t * 6 * NE;
        for (int m = 0; m < NOD; ++m) {
            // deriv = jac^-1 der (ascending k), BEEMAT rows ex, ey, ez, gxy, gyz, gzx
            double dd[3];
            for (int a = 0; a < 3; ++a) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += jac[a + 3 * k] * der[k + 3 * m];
                dd[a] = s;
            }
            const int l = 3 * m;   // columns l (x), l+1 (y), l+2 (z)
            for (int a = 0; a < 18; ++a) B[6 * l + a] = 0.0;
            B[0 + 6 * l] = dd[0];
            B[3 + 6 * l] = dd[1];
            B[5 + 6 * l] = dd[2];
            B[1 + 6 * (l + 1)] = dd[1];
            B[3 + 6 * (l + 1)] = dd[0];
            B[4 + 6 * (l + 1)] = dd[2];
            B[2 + 6 * (l + 2)] = dd[2];
            B[4 + 6 * (l + 2)] = dd[1];
            B[5 + 6 * (l + 2)] = dd[0];
        }
        detw[2 * t] = det;
        detw[2 * t + 1] = gp[4 * g + 3];
    }
}

// INVAR, nst = 6 (new_library.f90:1813-1916)
__device__ void invar6(const double *s, double &sigm, double &dsbar, double &theta)
{
    const double sq3 = sqrt(3.0);
    const double s1 = s[0], s2 = s[1], s3 = s[2], s4 = s[3], s5 = s[4], s6 = s[5];
    sigm = (s1 + s2 + s3) / 3.0;
    const double d2 = ((s1 - s2) * (s1 - s2) + (s2 - s3) * (s2 - s3) + (s3 - s1) * (s3 - s1)) / 6.0 + s4 * s4 +
                      s5 * s5 + s6 * s6;
    const double ds1 = s1 - sigm, ds2 = s2 - sigm, ds3 = s3 - sigm;
    const double d3 = ds1 * ds2 * ds3 - ds1 * s5 * s5 - ds2 * s6 * s6 - ds3 * s4 * s4 + 2.0 * s4 * s5 * s6;
    dsbar = sq3 * sqrt(d2);
    if (dsbar < 1.e-10) {
        theta = 0.0;
    } else {
        const double r = sqrt(d2);
        double sine = -3.0 * sq3 * d3 / (2.0 * (r * r * r));
        sine = sine > 1.0 ? 1.0 : (sine < -1.0 ? -1.0 : sine);
        theta = asin(sine) / 3.0;
    }
}

// One warp per element: the Gauss-point loop of p122.f90:172-202.  Lane l
// owns rows l and l+32 of the element vectors (rows below 3 NOD); every lane
// evaluates the point's scalar plasticity (the same values), lane 0 writes
// evpt / tensor.  bload = sum over points (in order) of B' devp det w, into
// ut[e * 3 NOD + k].
template <int NOD>
__global__ void __launch_bounds__(256)
k_p122_plastic(int nels, int nip, const int *__restrict__ conn, const double *__restrict__ loads,
               const double *__restrict__ bee, const double *__restrict__ detw, double *__restrict__ evpt,
               double *__restrict__ tensor, double phi, double c, double psi, double e, double v, double dt,
               int last, double *__restrict__ ut)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    // DEEMAT (new_library.f90:1671-1689)
    double d11, d12, d44;
    deemat3(e, v, d11, d12, d44);
    const double pi4 = 4.0 * atan(1.0);
    const double phir = phi * pi4 / 180.0, psir = psi * pi4 / 180.0;
    const double snph = sin(phir), csph = cos(phir), snps = sin(psir), sq3 = sqrt(3.0);
    constexpr int NE = 3 * NOD;
    const int k0 = lane, k1 = lane + 32;
    const bool h0 = k0 < NE, h1 = k1 < NE;   // the rows this lane holds
    for (int el = warp; el < nels; el += nwarps) {
        const int cn = lane < NOD ? conn[(size_t)el * NOD + lane] : 0;
        const int n0 = __shfl_sync(FULLMASK, cn, h0 ? k0 / 3 : 0);
        const int n1 = __shfl_sync(FULLMASK, cn, h1 ? k1 / 3 : 0);
        const double u0 = h0 ? loads[(size_t)3 * n0 + k0 % 3] : 0.0;
        const double u1 = h1 ? loads[(size_t)3 * n1 + k1 % 3] : 0.0;
        double bl0 = 0.0, bl1 = 0.0;
        for (int g = 0; g < nip; ++g) {
            const size_t gi = (size_t)el * nip + g;
            const double *B = bee + gi * 6 * NE;
            double eps[6];
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                double t = (h0 ? B[a + 6 * k0] * u0 : 0.0) + (h1 ? B[a + 6 * k1] * u1 : 0.0);
                eps[a] = warp_sum(t);
            }
            double *ev = evpt + gi * 6, *tn = tensor + gi * 6;
            double stress[6], sg[6];
#pragma unroll
            for (int a = 0; a < 6; ++a) eps[a] = eps[a] - ev[a];
            sg[0] = d11 * eps[0] + d12 * eps[1] + d12 * eps[2];
            sg[1] = d12 * eps[0] + d11 * eps[1] + d12 * eps[2];
            sg[2] = d12 * eps[0] + d12 * eps[1] + d11 * eps[2];
            sg[3] = d44 * eps[3];
            sg[4] = d44 * eps[4];
            sg[5] = d44 * eps[5];
#pragma unroll
            for (int a = 0; a < 6; ++a) stress[a] = sg[a] + tn[a];
            double sigm, dsbar, theta;
            invar6(stress, sigm, dsbar, theta);
            // MOCOUF (new_library.f90:2364-2417)
            const double csth = cos(theta), snth = sin(theta);
            const double f = snph * sigm + dsbar * (csth / sq3 - snth * snph / 3.0) - c * csph;
            double devp[6] = {0, 0, 0, 0, 0, 0};
            __syncwarp();   // every lane has read evpt / tensor of this point
            if (last) {
#pragma unroll
                for (int a = 0; a < 6; ++a) devp[a] = stress[a];
            } else if (f >= 0.0) {
                // MOCOUQ (new_library.f90:2423-2490)
                double dq1 = snps, dq2, dq3;
                if (fabs(snth) > 0.49) {
                    const double c1 = snth < 0.0 ? -1.0 : 1.0;
                    dq2 = (sq3 * 0.5 - c1 * snps * 0.5 / sq3) * sq3 * 0.5 / dsbar;
                    dq3 = 0.0;
                } else {
                    const double cs3th = cos(3.0 * theta), tn3th = tan(3.0 * theta), tnth = snth / csth;
                    dq2 = sq3 * csth / dsbar * ((1.0 + tnth * tn3th) + snps * (tn3th - tnth) / sq3) * 0.5;
                    dq3 = 0.5 * 3.0 * (sq3 * snth + snps * csth) / (cs3th * dsbar * dsbar);
                }
                // FORMM, nst = 6 (new_library.f90:85-198): flow = f (m1 dq1 + m2 dq2 + m3 dq3)
                const double sx = stress[0], sy = stress[1], sz = stress[2];
                const double txy = stress[3], tyz = stress[4], tzx = stress[5];
                const double sm = (sx + sy + sz) / 3.0, dx = sx - sm, dy = sy - sm, dz = sz - sm;
                double m1[36], m2[36], m3[36];
#pragma unroll
                for (int k = 0; k < 36; ++k) m1[k] = m2[k] = m3[k] = 0.0;
#define MM(m, i, j) m[((i) - 1) + 6 * ((j) - 1)]
                for (int i = 1; i <= 3; ++i)
                    for (int j = 1; j <= 3; ++j) MM(m1, i, j) = 1.0 / (3.0 * sm);
                for (int i = 1; i <= 3; ++i) {
                    MM(m2, i, i) = 2.0;
                    MM(m2, i + 3, i + 3) = 6.0;
                }
                MM(m2, 1, 2) = -1.0; MM(m2, 1, 3) = -1.0; MM(m2, 2, 3) = -1.0;
                MM(m3, 1, 1) = dx; MM(m3, 1, 2) = dz; MM(m3, 1, 3) = dy; MM(m3, 1, 4) = txy;
                MM(m3, 1, 5) = -2.0 * tyz; MM(m3, 1, 6) = tzx; MM(m3, 2, 2) = dy; MM(m3, 2, 3) = dx;
                MM(m3, 2, 4) = txy; MM(m3, 2, 5) = tyz; MM(m3, 2, 6) = -2.0 * tzx; MM(m3, 3, 3) = dz;
                MM(m3, 3, 4) = -2.0 * txy; MM(m3, 3, 5) = tyz; MM(m3, 3, 6) = tzx; MM(m3, 4, 4) = -3.0 * dz;
                MM(m3, 4, 5) = 3.0 * tzx; MM(m3, 4, 6) = 3.0 * tyz; MM(m3, 5, 5) = -3.0 * dx;
                MM(m3, 5, 6) = 3.0 * txy; MM(m3, 6, 6) = -3.0 * dy;
                for (int i = 1; i <= 6; ++i)
                    for (int j = i + 1; j <= 6; ++j) {
                        MM(m1, j, i) = MM(m1, i, j);
                        MM(m2, j, i) = MM(m2, i, j);
                        MM(m3, j, i) = MM(m3, i, j);
                    }
#undef MM
                double evp[6];
#pragma unroll
                for (int a = 0; a < 6; ++a) {
                    double s = 0.0;
                    for (int k = 0; k < 6; ++k) {
                        const double fl = f * (m1[a + 6 * k] / 3.0 * dq1 + m2[a + 6 * k] / 3.0 * dq2 +
                                               m3[a + 6 * k] / 3.0 * dq3);
                        s += fl * stress[k];
                    }
                    evp[a] = s * dt;
                }
                if (lane == 0)
                    for (int a = 0; a < 6; ++a) ev[a] = ev[a] + evp[a];
                devp[0] = d11 * evp[0] + d12 * evp[1] + d12 * evp[2];
                devp[1] = d12 * evp[0] + d11 * evp[1] + d12 * evp[2];
                devp[2] = d12 * evp[0] + d12 * evp[1] + d11 * evp[2];
                devp[3] = d44 * evp[3];
                devp[4] = d44 * evp[4];
                devp[5] = d44 * evp[5];
            }
            if (f >= 0.0) {
                const double dw = detw[2 * gi], w = detw[2 * gi + 1];
                double s0 = 0.0, s1 = 0.0;
#pragma unroll
                for (int a = 0; a < 6; ++a) {
                    if (h0) s0 += B[a + 6 * k0] * devp[a];
                    if (h1) s1 += B[a + 6 * k1] * devp[a];
                }
                bl0 = bl0 + s0 * dw * w;
                bl1 = bl1 + s1 * dw * w;
            }
            if (last && lane == 0)
                for (int a = 0; a < 6; ++a) tn[a] = stress[a];
        }
        if (h0) ut[(size_t)el * NE + k0] = bl0;
        if (h1) ut[(size_t)el * NE + k1] = bl1;
    }
}

// The load vector of a plastic iteration (p122.f90:121-140), over slots:
// with nodal loads, loads = ld0 * q + bdylds; without, loads = bdylds, or 0
// on the first plastic iteration (first != 0).
__global__ void k_p122_loads(int ns, const double *__restrict__ ld0, double q, const double *__restrict__ bdylds,
                             int first, double *__restrict__ loads)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x)
        loads[s] = ld0 ? ld0[s] * q + bdylds[s] : (first ? 0.0 : bdylds[s]);
}

// fixed freedoms (p122.f90:122-139): on the first plastic iteration
// loads = store * value * q, after it loads = 0
__global__ void k_p122_fixed_loads(int nfix, const int *__restrict__ slot, const double *__restrict__ val,
                                   const double *__restrict__ fstore, double q, int first, double *__restrict__ loads)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nfix; i += gridDim.x * blockDim.x) {
        const int s = slot[i];
        loads[s] = first ? fstore[s] * val[i] * q : 0.0;
    }
}

// checon_par on (x, oldis): block partials of max|x| and max|x - oldis|; oldis = x
__global__ void __launch_bounds__(256)
k_p122_checon(int ns, const double *__restrict__ x, double *__restrict__ oldis, double *__restrict__ part, int G)
{
    double ml = 0.0, md = 0.0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const double xv = x[s];
        ml = fmax(ml, fabs(xv));
        md = fmax(md, fabs(xv - oldis[s]));
        oldis[s] = xv;
    }
    double v[2] = {ml, md};
    block_reduce<2>(v, 3u);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = v[0];
        part[G + blockIdx.x] = v[1];
    }
}

__global__ void k_p122_checon2(const double *__restrict__ part, int G, double *__restrict__ out)
{
    const double ml = reduce_partials(part, G, true);
    const double md = reduce_partials(part + G, G, true);
    if (threadIdx.x == 0) {
        out[0] = ml;
        out[1] = md;
    }
}

__global__ void k_p122_add(int ns, double *__restrict__ y, const double *__restrict__ x)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) y[s] = y[s] + x[s];
}

}  // namespace pf

using namespace pf;

#define PCK(call)                                                                        \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            p122_free(q);                                                                \
            return PF_FAILURE;                                                           \
        }                                                                                \
    } while (0)
#define PTRY(call)              \
    do {                        \
        if (call) {             \
            p122_free(q);       \
            return PF_FAILURE;  \
        }                       \
    } while (0)

namespace pf {
int run_pcg_public(Ctx &c, int prec, double *xsol, int limit);   // pf_abi.cu: PCG iterations until the state stops
}

static int p122_launched(Ctx &c, const char *name)
{
    c.launches++;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: launch failed: %s", name, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

extern "C" int pf_p122_solve_fixed(void **ctx, const int *nip, const double *phi, const double *c_coh,
                                   const double *psi, const int *incs, const double *qinc, const int *plasits,
                                   const int *cjits, const double *plastol, const double *cjtol, const double *ld0,
                                   const int *nfix_p, const int *fix_eqs, const double *fix_vals, double *results,
                                   double *totd_out, int *incs_done)
try {
    if (!ctx || !*ctx || !nip || !phi || !c_coh || !psi || !incs || !qinc || !plasits || !cjits || !plastol ||
        !cjtol || !nfix_p || !results || !incs_done) {
        set_error("pf_p122_solve: null argument");
        return PF_FAILURE;
    }
    Ctx &c = *(Ctx *)*ctx;
    if (cudaSetDevice(c.device) != cudaSuccess) {
        set_error("pf_p122_solve: cannot select the device");
        return PF_FAILURE;
    }
    const int nfix = *nfix_p;
    if ((c.kind != KIND_SOLID20 && c.kind != KIND_SOLID8) || c.shared || !c.have_km || !c.km64 || c.nmat != 1 ||
        *incs < 1 || *plasits < 1 || *cjits < 1 || (*nip != 8 && *nip != 27) || nfix < 0 ||
        (nfix > 0 && (!fix_eqs || !fix_vals)) || (nfix == 0 && !ld0)) {
        set_error("pf_p122_solve: needs an elasticity context with storkm formed from one material, incs, "
                  "plasits, cjits >= 1, nip 8 or 27, and nodal loads or fixed freedoms");
        return PF_FAILURE;
    }
    if (nfix > 0 && c.kind != KIND_SOLID8) {
        set_error("pf_p122_solve: fixed freedoms need an 8-node context (pf_setup_solid8)");
        return PF_FAILURE;
    }
    const bool solid8 = c.kind == KIND_SOLID8;
    const int ne = solid8 ? 24 : 60;
    P122 q;
    q.nip = *nip;
    const size_t ns = c.nslots, ngp = (size_t)c.nels * q.nip;
    PCK(cudaMalloc(&q.bee, ngp * 6 * ne * sizeof(double)));
    PCK(cudaMalloc(&q.detw, ngp * 2 * sizeof(double)));
    PCK(cudaMalloc(&q.evpt, ngp * 6 * sizeof(double)));
    PCK(cudaMalloc(&q.tensor, ngp * 6 * sizeof(double)));
    double **vecs[] = {&q.loads, &q.bdylds, &q.oldis, &q.totd};
    for (double **v : vecs) PCK(cudaMalloc(v, ns * sizeof(double)));
    PCK(cudaMalloc(&q.red, (2 * (size_t)c.G + 8) * sizeof(double)));
    PCK(cudaMemsetAsync(q.tensor, 0, ngp * 6 * sizeof(double), c.stream));
    PCK(cudaMemsetAsync(q.oldis, 0, ns * sizeof(double), c.stream));
    PCK(cudaMemsetAsync(q.totd, 0, ns * sizeof(double), c.stream));
    PCK(cudaMemsetAsync(c.x, 0, ns * sizeof(double), c.stream));
    if (ld0) {   // ld0 to slots
        PCK(cudaMalloc(&q.ld0, ns * sizeof(double)));
        PCK(cudaMemcpyAsync(c.eqbuf, ld0, (size_t)c.neq * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        PTRY(launch_eq_to_slot(c, c.eqbuf, q.ld0));
    }
    if (nfix > 0) {
        // the penalty on the fixed freedoms' diagonal, store = the penalised
        // diagonal (p122.f90:108-113)
        std::vector<int> eq_slot(c.neq), slots(nfix);
        PCK(cudaMemcpy(eq_slot.data(), c.eq_slot, (size_t)c.neq * sizeof(int), cudaMemcpyDeviceToHost));
        for (int i = 0; i < nfix; ++i) {
            if (fix_eqs[i] < 1 || fix_eqs[i] > c.neq) {
                set_error("pf_p122_solve: fixed freedom %d: equation %d outside 1..%d", i + 1, fix_eqs[i], c.neq);
                p122_free(q);
                return PF_FAILURE;
            }
            slots[i] = eq_slot[fix_eqs[i] - 1];
        }
        PCK(cudaMalloc(&q.fslot, nfix * sizeof(int)));
        PCK(cudaMalloc(&q.fval, nfix * sizeof(double)));
        PCK(cudaMemcpyAsync(q.fslot, slots.data(), nfix * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        PCK(cudaMemcpyAsync(q.fval, fix_vals, nfix * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        PTRY(launch_set_fixed(c, nfix, q.fslot, 1.e20));
    }
    // B, det, w at every Gauss point
    double *gp = nullptr;
    PCK(cudaMalloc(&gp, sizeof(double) * 4 * 27));
    if (launch_sample(c.stream, q.nip, false, gp)) {
        cudaFree(gp);
        p122_free(q);
        return PF_FAILURE;
    }
    if (solid8)
        k_p122_bee<8><<<c.nsm * 8, 128, 0, c.stream>>>(c.nels, q.nip, gp, c.coord, q.bee, q.detw);
    else
        k_p122_bee<20><<<c.nsm * 8, 128, 0, c.stream>>>(c.nels, q.nip, gp, c.coord, q.bee, q.detw);
    if (p122_launched(c, "k_p122_bee")) {
        cudaFree(gp);
        p122_free(q);
        return PF_FAILURE;
    }
    PCK(cudaStreamSynchronize(c.stream));
    cudaFree(gp);
    double e = 0.0, v = 0.0;
    PCK(cudaMemcpy(&e, c.mat_e, sizeof(double), cudaMemcpyDeviceToHost));
    PCK(cudaMemcpy(&v, c.mat_v, sizeof(double), cudaMemcpyDeviceToHost));
    const double pi = std::acos(-1.0), snph = std::sin(*phi * pi / 180.0);
    const double dt = 4.0 * (1.0 + v) * (1.0 - 2.0 * v) / (e * (1.0 - 2.0 * v + snph * snph));
    const int gv = c.G, ge = c.nels < c.nsm * 64 ? (c.nels + 7) / 8 : c.nsm * 8;
    static const double kOne = 1.0, kZero = 0.0;
    // slot of equation 1 for the printed displacement
    int slot1 = -1;
    if (c.neq > 0) PCK(cudaMemcpy(&slot1, c.eq_slot, sizeof(int), cudaMemcpyDeviceToHost));
    int iy = 0;
    for (iy = 1; iy <= *incs; ++iy) {
        int plasiters = 0, cjtot = 0;
        PCK(cudaMemsetAsync(q.bdylds, 0, ns * sizeof(double), c.stream));
        PCK(cudaMemsetAsync(q.evpt, 0, ngp * 6 * sizeof(double), c.stream));
        for (;;) {
            ++plasiters;
            const int first = plasiters == 1 ? 1 : 0;
            k_p122_loads<<<gv, 256, 0, c.stream>>>((int)ns, q.ld0, qinc[iy - 1], q.bdylds, first, q.loads);
            PTRY(p122_launched(c, "k_p122_loads"));
            if (nfix > 0 && !(first && ld0)) {   // with nodal loads the first iteration's vector replaces them
                k_p122_fixed_loads<<<1, 256, 0, c.stream>>>(nfix, q.fslot, q.fval, c.fstore, qinc[iy - 1], first,
                                                            q.loads);
                PTRY(p122_launched(c, "k_p122_fixed_loads"));
            }
            if (solid8)   // the product at a fixed freedom: p * store on the first iteration, 0 after
                PCK(cudaMemcpyAsync(c.fscale, first ? &kOne : &kZero, sizeof(double), cudaMemcpyHostToDevice,
                                    c.stream));
            // r = loads - K x (warm start from the previous solution), then PCG with checon_par
            PTRY(launch_residual(c, q.loads, c.x, c.rres));
            PTRY(launch_pcg_init(c, c.rres, c.x, STOP_CHECON, *cjtol, *cjits, true));
            PTRY(run_pcg_public(c, 64, c.x, *cjits));
            cjtot += c.hst->iters;
            // loads = xnew; plastic checon against oldis
            PCK(cudaMemcpyAsync(q.loads, c.x, ns * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
            k_p122_checon<<<gv, 256, 0, c.stream>>>((int)ns, q.loads, q.oldis, q.red, gv);
            PTRY(p122_launched(c, "k_p122_checon"));
            k_p122_checon2<<<1, 256, 0, c.stream>>>(q.red, gv, q.red + 2 * gv);
            PTRY(p122_launched(c, "k_p122_checon2"));
            double mx[2] = {0, 0};
            PCK(cudaMemcpyAsync(mx, q.red + 2 * gv, 2 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            PCK(cudaStreamSynchronize(c.stream));
            const bool conv = plasiters > 1 && mx[1] / mx[0] <= *plastol;
            const bool last = conv || plasiters == *plasits;
            if (last) PCK(cudaMemsetAsync(q.bdylds, 0, ns * sizeof(double), c.stream));
            if (solid8)
                k_p122_plastic<8><<<ge, 256, 0, c.stream>>>(c.nels, q.nip, c.conn, q.loads, q.bee, q.detw, q.evpt,
                                                            q.tensor, *phi, *c_coh, *psi, e, v, dt, last ? 1 : 0,
                                                            (double *)c.utemp);
            else
                k_p122_plastic<20><<<ge, 256, 0, c.stream>>>(c.nels, q.nip, c.conn, q.loads, q.bee, q.detw, q.evpt,
                                                             q.tensor, *phi, *c_coh, *psi, e, v, dt, last ? 1 : 0,
                                                             (double *)c.utemp);
            PTRY(p122_launched(c, "k_p122_plastic"));
            PTRY(launch_scatter_add64(c, q.bdylds));
            if (last) break;
        }
        k_p122_add<<<gv, 256, 0, c.stream>>>((int)ns, q.totd, q.loads);
        PTRY(p122_launched(c, "k_p122_add"));
        double *o = results + 6 * (iy - 1);
        double t1 = 0.0, tn[6];
        if (slot1 >= 0) PCK(cudaMemcpyAsync(&t1, q.totd + slot1, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        PCK(cudaMemcpyAsync(tn, q.tensor, 6 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if (totd_out) {
            PTRY(launch_slot_to_eq(c, q.totd, c.eqbuf));
            PCK(cudaMemcpyAsync(totd_out + (size_t)c.neq * (iy - 1), c.eqbuf, (size_t)c.neq * sizeof(double),
                                cudaMemcpyDeviceToHost, c.stream));
        }
        PCK(cudaStreamSynchronize(c.stream));
        o[0] = t1;
        o[1] = tn[2];
        o[2] = tn[0];
        o[3] = tn[1];
        o[4] = cjtot;
        o[5] = plasiters;
        if (plasiters == *plasits) break;
    }
    *incs_done = iy > *incs ? *incs : iy;
    if (nfix > 0) {   // the context's diagonal without the penalties, no fixed freedoms
        PTRY(launch_assemble_diag(c));
        PCK(cudaMemsetAsync(c.fstore, 0, ns * sizeof(double), c.stream));
    }
    if (solid8) PCK(cudaMemcpyAsync(c.fscale, &kOne, sizeof(double), cudaMemcpyHostToDevice, c.stream));
    PCK(cudaStreamSynchronize(c.stream));
    p122_free(q);
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_p122_solve_fixed");
}

extern "C" int pf_p122_solve(void **ctx, const int *nip, const double *phi, const double *c_coh, const double *psi,
                             const int *incs, const double *qinc, const int *plasits, const int *cjits,
                             const double *plastol, const double *cjtol, const double *ld0, double *results,
                             double *totd_out, int *incs_done)
try {
    if (!ld0) {
        set_error("pf_p122_solve: null argument");
        return PF_FAILURE;
    }
    const int zero = 0;
    return pf_p122_solve_fixed(ctx, nip, phi, c_coh, psi, incs, qinc, plasits, cjits, plastol, cjtol, ld0, &zero,
                               nullptr, nullptr, results, totd_out, incs_done);
} catch (...) {
    return pf::host_exception("pf_p122_solve");
}
