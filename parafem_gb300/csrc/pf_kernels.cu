// pf_kernels.cu -- sm_103a kernels of the element-by-element PCG path.
//
// Layout on the device (one context):
//   vectors are node-major "slots": slot 3*n+d is dof d of node n (0-based);
//   restrained slots hold 0, which plays the role of p121's equation 0
//   (GATHER sets pl(0)=0, SCATTER drops contributions to it,
//   src/modules/mpi/gather_scatter.f90:547-854).
//   storkm(60,60,e) keeps p121's column-major element blocks.
// Reductions are deterministic: fixed per-thread assignment, xor-shuffle
// trees, per-block partials summed in a fixed order by the consumer kernel.
#include "pf_device.cuh"
#include "pf_tc.cuh"

#include <cmath>
#include <cstdio>

namespace pf {

static int check_launch(Ctx &c, const char *name)
{
    c.launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: launch failed: %s", name, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// SAMPLE (src/modules/shared/new_library.f90:1397-1514), nip 8 or 27.
// gp[4*i] = (xi, eta, zeta, w).
__global__ void k_sample(int nip, int exact, double *gp)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double root3 = 1.0 / sqrt(3.0);
    const double r15 = 0.2 * sqrt(15.0);
    if (nip == 8) {
        const int sg[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                              {-1, 1, 1}, {-1, -1, 1}, {-1, 1, -1}, {-1, -1, -1}};
        for (int i = 0; i < 8; ++i) {
            for (int d = 0; d < 3; ++d) gp[4 * i + d] = sg[i][d] * root3;
            gp[4 * i + 3] = 1.0;
        }
    } else if (nip == 27) {
        const double w3[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
        double v9[9];
        for (int i = 0; i < 3; ++i) {
            v9[i] = 5.0 / 9.0 * w3[i];
            v9[3 + i] = 8.0 / 9.0 * w3[i];
            v9[6 + i] = 5.0 / 9.0 * w3[i];
        }
        // p121 takes 5./9. and 8./9. as default-REAL literals (:1493)
        const double f59 = exact ? 5.0 / 9.0 : (double)(5.0f / 9.0f);
        const double f89 = exact ? 8.0 / 9.0 : (double)(8.0f / 9.0f);
        for (int blk = 0; blk < 3; ++blk) {
            const double eta = blk == 0 ? -r15 : (blk == 1 ? 0.0 : r15);
            const double f = blk == 1 ? f89 : f59;
            for (int i = 0; i < 9; ++i) {
                const int col = i % 3, row = i / 3;
                double *g = &gp[4 * (blk * 9 + i)];
                g[0] = col == 0 ? -r15 : (col == 1 ? 0.0 : r15);
                g[1] = eta;
                g[2] = row == 0 ? r15 : (row == 1 ? 0.0 : -r15);
                g[3] = f * v9[i];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// storkm integration (p121.f90:54-64): sum over the Gauss points of
// B'DB*det*w.  For isotropic D and nodes a, b with gradients ga, gb the 3x3
// block of B'DB is
//   (i,i): D11 ga_i gb_i + D44 sum_{k!=i} ga_k gb_k
//   (i,j): D12 ga_i gb_j + D44 ga_j gb_i
// -- the dense MATMUL(MATMUL(TRANSPOSE(bee),dee),bee) of p121.f90:61-62 with
// the zero entries of bee (BEEMAT, new_library.f90:976-993) skipped.  Both
// are linear in M_ab(i,j) = sum_gp det*w ga_i gb_j, so each node pair
// accumulates M_ab (9 FMA per point) and forms its block once.
//
// One CTA of kFormThreads threads per element (grid-stride): the shape
// derivatives at the Gauss points are computed once per CTA; per element the
// 27 Jacobians, their inverses and the 27 x 20 gradients are formed in four
// phases, then thread t < 210 owns node pair (a, b), a <= b, and writes the
// blocks (a, b) and (b, a) = (a, b)'.  GB300's FP64 rate is about 1/60 of its
// FP32 rate; this order needs about 64k FP64 operations per element at
// nip = 27 instead of the 486k of a per-point B'DB.
// The same for 8-node bricks (NOD = 8: 36 node pairs, 24 x 24 storkm).
constexpr int kFormThreads = 224;
template <int NOD>
__global__ void __launch_bounds__(kFormThreads)
k_form_storkm(int nels, int nip, const double *__restrict__ gp, const double *__restrict__ coord,
              const double *__restrict__ me, const double *__restrict__ mv, int nmat,
              double *__restrict__ km64, float *__restrict__ km32, double *__restrict__ ediag)
{
    constexpr int NE = 3 * NOD, NP = NOD * (NOD + 1) / 2;
    __shared__ double s_der[27][NE];   // der(3,NOD) at each point
    __shared__ double s_w[27];
    __shared__ double s_coord[NE];     // coord(NOD,3)
    __shared__ double s_jac[27][9];    // jac, then its inverse
    __shared__ double s_wd[27];        // det * w
    __shared__ double s_g[27][NE];     // deriv(3,NOD) = jac^-1 der
    __shared__ double s_h[27][NE];     // det * w * deriv
    __shared__ double s_D[3];
    const int t = threadIdx.x;
    for (int k = t; k < nip * NOD; k += kFormThreads) {
        const int ig = k / NOD, l = k % NOD;
        if constexpr (NOD == 20) shape_der20(l, gp[4 * ig], gp[4 * ig + 1], gp[4 * ig + 2], &s_der[ig][3 * l]);
        else shape_der8(l, gp[4 * ig], gp[4 * ig + 1], gp[4 * ig + 2], &s_der[ig][3 * l]);
        if (l == 0) s_w[ig] = gp[4 * ig + 3];
    }
    // this thread's node pair: t = b(b+1)/2 + a, a <= b
    int pa = 0, pb = 0;
    if (t < NP) {
        while ((pb + 1) * (pb + 2) / 2 <= t) ++pb;
        pa = t - pb * (pb + 1) / 2;
    }
    for (int e = blockIdx.x; e < nels; e += gridDim.x) {
        if (t < NE) s_coord[t] = coord[(size_t)e * NE + t];
        if (t == 0) {
            const int m = nmat == 1 ? 0 : e;
            deemat3(me[m], mv[m], s_D[0], s_D[1], s_D[2]);
        }
        __syncthreads();
        for (int k = t; k < nip * 9; k += kFormThreads) {   // jac = MATMUL(der, coord)
            const int ig = k / 9, a = k % 3, b = (k / 3) % 3;
            double s = 0.0;
            for (int n = 0; n < NOD; ++n) s += s_der[ig][a + 3 * n] * s_coord[n + NOD * b];
            s_jac[ig][a + 3 * b] = s;
        }
        __syncthreads();
        if (t < nip) s_wd[t] = det_invert3(s_jac[t]) * s_w[t];
        __syncthreads();
        for (int k = t; k < nip * NE; k += kFormThreads) {   // deriv = MATMUL(jac^-1, der)
            const int ig = k / NE, a = k % 3, l = (k / 3) % NOD;
            const double *j = s_jac[ig];
            const double g = j[a] * s_der[ig][3 * l] + j[a + 3] * s_der[ig][1 + 3 * l] + j[a + 6] * s_der[ig][2 + 3 * l];
            s_g[ig][a + 3 * l] = g;
            s_h[ig][a + 3 * l] = s_wd[ig] * g;
        }
        __syncthreads();
        if (t < NP) {
            double M[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) M[k] = 0.0;
            for (int ig = 0; ig < nip; ++ig) {
                const double ha0 = s_h[ig][3 * pa], ha1 = s_h[ig][3 * pa + 1], ha2 = s_h[ig][3 * pa + 2];
                const double gb0 = s_g[ig][3 * pb], gb1 = s_g[ig][3 * pb + 1], gb2 = s_g[ig][3 * pb + 2];
                M[0] = fma(ha0, gb0, M[0]); M[1] = fma(ha1, gb0, M[1]); M[2] = fma(ha2, gb0, M[2]);
                M[3] = fma(ha0, gb1, M[3]); M[4] = fma(ha1, gb1, M[4]); M[5] = fma(ha2, gb1, M[5]);
                M[6] = fma(ha0, gb2, M[6]); M[7] = fma(ha1, gb2, M[7]); M[8] = fma(ha2, gb2, M[8]);
            }
            const double D11 = s_D[0], D12 = s_D[1], D44 = s_D[2];
            double K[9];   // K(i + 3j) of block (a, b); M(i + 3j) = sum det w ga_i gb_j
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    if (i == j) {
                        const int k1 = (i + 1) % 3, k2 = (i + 2) % 3;
                        K[i + 3 * j] = D11 * M[i + 3 * i] + D44 * (M[k1 + 3 * k1] + M[k2 + 3 * k2]);
                    } else {
                        K[i + 3 * j] = D12 * M[i + 3 * j] + D44 * M[j + 3 * i];
                    }
                }
            double *ke = km64 ? km64 + (size_t)e * NE * NE : nullptr;
            float *kf = km32 ? km32 + (size_t)e * NE * NE : nullptr;
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const double v = K[i + 3 * j];
                    const int ab = (3 * pb + j) * NE + 3 * pa + i, ba = (3 * pa + i) * NE + 3 * pb + j;
                    if (ke) {
                        ke[ab] = v;
                        if (pa != pb) ke[ba] = v;
                    }
                    if (kf) {
                        kf[ab] = (float)v;
                        if (pa != pb) kf[ba] = (float)v;
                    }
                    if (pa == pb && i == j) ediag[(size_t)e * NE + 3 * pa + i] = v;
                }
        }
        __syncthreads();
    }
}

__global__ void k_cast_km32(size_t n, const double *__restrict__ a, float *__restrict__ b)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void k_extract_ediag(int nels, const double *__restrict__ km, double *__restrict__ ed)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)nels * 60;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t e = i / 60, k = i % 60;
        ed[i] = km[e * 3600 + k * 61];
    }
}

// Jacobi diagonal (p121.f90:65-69, 86): node-centric sum of element
// diagonals in ascending element order -- the order of the serial SCATTER.
__global__ void k_assemble_diag(int nn, const int *__restrict__ ptr, const int *__restrict__ list,
                                const double *__restrict__ ed, const uint8_t *__restrict__ fm,
                                double *__restrict__ diag, double *__restrict__ dinv)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += gridDim.x * blockDim.x) {
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int k = ptr[n]; k < ptr[n + 1]; ++k) {
            const double *q = ed + (size_t)list[k] * 3;
            a0 += q[0];
            a1 += q[1];
            a2 += q[2];
        }
        const int m = fm[n];
        const double a[3] = {a0, a1, a2};
        for (int d = 0; d < 3; ++d) {
            const bool fr = (m >> d) & 1;
            diag[3 * n + d] = fr ? a[d] : 0.0;
            dinv[3 * n + d] = fr ? 1.0 / a[d] : 0.0;
        }
    }
}

// ---------------------------------------------------------------------------
// Element products (p121.f90:92-97): one warp per element.  Lanes 0..19
// fetch the connectivity, every lane gathers p for dofs lane and lane+32,
// lanes 0..29 then own rows 2*lane and 2*lane+1 and walk the 60 columns of
// storkm(:,:,e) with 2-wide loads, p(j) broadcast by shuffle.
template <typename KT> struct Vec2;
template <> struct Vec2<double> { typedef double2 T; };
template <> struct Vec2<float> { typedef float2 T; };

// One element's product by one warp (the body of k_elem, shared with the
// persistent FP64 iteration kernel).
template <typename KT, bool GATHER>
__device__ __forceinline__ void elem_warp(int e, int lane, const KT *__restrict__ km, const int *__restrict__ conn,
                                          const double *__restrict__ p, KT *__restrict__ ut)
{
    typedef typename Vec2<KT>::T V2;
    const int j1 = lane + 32;
    KT p0, p1;
    if (GATHER) {
        const int nd = (lane < 20) ? conn[(size_t)e * 20 + lane] : 0;
        const int n0 = __shfl_sync(FULLMASK, nd, lane / 3);
        const int n1 = __shfl_sync(FULLMASK, nd, j1 < 60 ? j1 / 3 : 0);
        p0 = (KT)p[(size_t)3 * n0 + lane % 3];
        p1 = (j1 < 60) ? (KT)p[(size_t)3 * n1 + j1 % 3] : (KT)0;
    } else {
        p0 = (KT)p[(size_t)e * 60 + lane];
        p1 = (j1 < 60) ? (KT)p[(size_t)e * 60 + j1] : (KT)0;
    }
    const KT *ke = km + (size_t)e * 3600 + 2 * lane;
    KT a0 = 0, a1 = 0;
#pragma unroll 12
    for (int j = 0; j < 60; ++j) {
        const KT pj = __shfl_sync(FULLMASK, j < 32 ? p0 : p1, j & 31);
        if (lane < 30) {
            const V2 k2 = __ldg(reinterpret_cast<const V2 *>(ke + 60 * j));
            a0 = fma(k2.x, pj, a0);
            a1 = fma(k2.y, pj, a1);
        }
    }
    if (lane < 30) {
        if constexpr (sizeof(KT) == 4) {   // FP32 results, node-padded: row i at (i/3)*4 + i%3
            const int i0 = 2 * lane, i1 = 2 * lane + 1;
            ut[(size_t)e * 80 + (i0 / 3) * 4 + i0 % 3] = a0;
            ut[(size_t)e * 80 + (i1 / 3) * 4 + i1 % 3] = a1;
        } else {
            V2 o;
            o.x = a0;
            o.y = a1;
            reinterpret_cast<V2 *>(ut + (size_t)e * 60)[lane] = o;
        }
    }
}

template <typename KT, bool GATHER>
__global__ void __launch_bounds__(256)
k_elem(int nels, const KT *__restrict__ km, const int *__restrict__ conn,
       const double *__restrict__ p, KT *__restrict__ ut, const PcgState *__restrict__ st)
{
    if (st && st->stop) return;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int e = warp; e < nels; e += nwarps) elem_warp<KT, GATHER>(e, lane, km, conn, p, ut);
}

// Node-centric scatter (SCATTER, gather_scatter.f90:694-854, one rank):
// each node sums its (element, local node) contributions in ascending
// element order, so the sum order equals the serial p121 SCATTER and runs
// are bitwise reproducible without atomics.  list[] holds contribution
// indices e*20+a.  FP64 results are read as three doubles at (e*20+a)*3;
// FP32 results are node-padded, so one 16-byte load fetches a contribution,
// and they are summed in FP32 (the precision of the products themselves).
// Contributions are fetched eight at a time so that a node's loads are in
// flight together.
//   MODE 0: out = u (restrained 0), partial p.u       (pf = p)
//   MODE 1: out = f - u (restrained 0), partial out.out (pf = f)
//   MODE 2: out += u at free dofs, no partials          (pf unused)
// One (virtual) block vb of nvb of the scatter: the body of k_scatter,
// shared with the persistent iteration kernels, which run the same blocks
// so that every partial sum is formed in the same order.  NC: the element
// results may be read through the non-coherent path (they were written by an
// earlier launch).  PF contributions are fetched at a time; the sums are
// formed in ascending order whatever PF is.
template <typename UT, int MODE, bool NC, int PF = 8>
__device__ __forceinline__ void scatter_block(int vb, int nvb, int nn, const int *__restrict__ ptr,
                                              const int *__restrict__ list, const UT *__restrict__ ut,
                                              const uint8_t *__restrict__ fm, const double *__restrict__ pf,
                                              double *__restrict__ out, double *__restrict__ part)
{
    double loc = 0.0;
    for (int n = vb * blockDim.x + threadIdx.x; n < nn; n += nvb * blockDim.x) {
        UT a0 = 0, a1 = 0, a2 = 0;
        const int k1 = ptr[n + 1];
        for (int k = ptr[n]; k < k1; k += PF) {
            int ci[PF];
#pragma unroll
            for (int i = 0; i < PF; ++i) ci[i] = (k + i < k1) ? __ldg(list + k + i) : -1;
            if constexpr (sizeof(UT) == 4) {
                float4 v[PF];
#pragma unroll
                for (int i = 0; i < PF; ++i)
                    if (ci[i] >= 0)
                        v[i] = NC ? __ldg(reinterpret_cast<const float4 *>(ut) + ci[i])
                                  : __ldcg(reinterpret_cast<const float4 *>(ut) + ci[i]);
#pragma unroll
                for (int i = 0; i < PF; ++i)
                    if (ci[i] >= 0) {
                        a0 += v[i].x;
                        a1 += v[i].y;
                        a2 += v[i].z;
                    }
            } else {
                double v[PF][3];
#pragma unroll
                for (int i = 0; i < PF; ++i)
                    if (ci[i] >= 0) {
                        const double *q = ut + (size_t)ci[i] * 3;
                        v[i][0] = NC ? q[0] : __ldcg(q);
                        v[i][1] = NC ? q[1] : __ldcg(q + 1);
                        v[i][2] = NC ? q[2] : __ldcg(q + 2);
                    }
#pragma unroll
                for (int i = 0; i < PF; ++i)
                    if (ci[i] >= 0) {
                        a0 += v[i][0];
                        a1 += v[i][1];
                        a2 += v[i][2];
                    }
            }
        }
        const int m = fm[n];
        const double a[3] = {(double)a0, (double)a1, (double)a2};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const size_t s = (size_t)3 * n + d;
            const bool fr = (m >> d) & 1;
            if (MODE == 0) {
                const double uv = fr ? a[d] : 0.0;
                out[s] = uv;
                loc = fma(pf[s], uv, loc);
            } else if (MODE == 1) {
                const double rv = fr ? pf[s] - a[d] : 0.0;
                out[s] = rv;
                loc = fma(rv, rv, loc);
            } else {   // MODE 2: out += sum (SCATTER's accumulation into an existing vector)
                if (fr) out[s] = out[s] + a[d];
            }
        }
    }
    if (MODE == 2) return;   // no partial sums (the kernel has no block barrier after this point)
    double v[1] = {loc};
    block_reduce<1>(v, 0u);
    if (threadIdx.x == 0) part[vb] = v[0];
}

template <typename UT, int MODE>
__global__ void __launch_bounds__(256)
k_scatter(int nn, const int *__restrict__ ptr, const int *__restrict__ list,
          const UT *__restrict__ ut, const uint8_t *__restrict__ fm, const double *__restrict__ pf,
          double *__restrict__ out, double *__restrict__ part, const PcgState *__restrict__ st)
{
    if (block_stopped(st)) return;
    scatter_block<UT, MODE, true>(blockIdx.x, gridDim.x, nn, ptr, list, ut, fm, pf, out, part);
}

// ---------------------------------------------------------------------------
// PCG (p121.f90:86-104).
// init: x = 0, r = rhs, d = dinv*r, p = d; partials r.d and r.r.  ps
// (shared-km contexts): the FP32 high and low parts of p, which the
// tensor-core product gathers instead of p.
__global__ void __launch_bounds__(256)
k_pcg_init(int ns, const double *__restrict__ rhs, const double *__restrict__ dinv,
           double *__restrict__ x, double *__restrict__ r, double *__restrict__ d,
           double *__restrict__ p, double *__restrict__ part, int G, int keep_x, float2 *__restrict__ ps)
{
    double rd = 0.0, rr = 0.0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const double rv = rhs[s];
        const double dv = dinv[s] * rv;
        if (!keep_x) x[s] = 0.0;
        r[s] = rv;
        d[s] = dv;
        p[s] = dv;
        if (ps) {
            float h, l;
            tc::split_f64(dv, h, l);
            ps[s] = make_float2(h, l);
        }
        rd = fma(rv, dv, rd);
        rr = fma(rv, rv, rr);
    }
    double v[2] = {rd, rr};
    block_reduce<2>(v, 0u);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = v[0];
        part[G + blockIdx.x] = v[1];
    }
}

__global__ void k_pcg_init2(PcgState *st, const double *__restrict__ part, int G, int stop_mode,
                            double tol, int limit)
{
    const double rd = reduce_partials(part, G, false);
    const double rr = reduce_partials(part + G, G, false);
    if (threadIdx.x == 0) {
        st->up = rd;
        st->ff = rr;
        st->rr = rr;
        st->metric = 0.0;
        st->tol = tol;
        st->iters = 0;
        st->converged = 0;
        st->limit = limit;
        st->stop_mode = stop_mode;
        st->err = 0;
        // a zero load vector is already solved by x = 0
        st->stop = (rr == 0.0) ? 1 : 0;
        if (rr == 0.0) st->converged = 1;
    }
}

// update1: alpha = up/(p.u); xnew = x + p*alpha (in place, checon_par's
// x = xnew, maths.f90:1062); r = r - u*alpha; d = diag*r; block partials of
// r.d, r.r and, for checon_par only (CHECON), max|xnew| and max|xnew-x|,
// into pu[0..4G).  p.u comes from the scatter's Gs partials ps.  Reads
// st->up only.  The max terms cost four FP64 operations per dof, a slow pipe
// on GB300, so the residual-stopped runs skip them.
template <bool CHECON>
__device__ __forceinline__ void update1_block(int vb, int nvb, int ns, double alpha, double *__restrict__ pu_out,
                                              int G, double *__restrict__ x, double *__restrict__ r,
                                              double *__restrict__ d, const double *__restrict__ p,
                                              const double *__restrict__ u, const double *__restrict__ dinv)
{
    double rd = 0.0, rr = 0.0, mx = 0.0, md = 0.0;
    for (int s = vb * blockDim.x + threadIdx.x; s < ns; s += nvb * blockDim.x) {
        const double xo = x[s];
        const double xn = fma(p[s], alpha, xo);
        x[s] = xn;
        if (CHECON) {
            mx = fmax(mx, fabs(xn));
            md = fmax(md, fabs(xn - xo));
        }
        const double rn = fma(-u[s], alpha, r[s]);
        r[s] = rn;
        const double dn = dinv[s] * rn;
        d[s] = dn;
        rd = fma(rn, dn, rd);
        rr = fma(rn, rn, rr);
    }
    double v[4] = {rd, rr, mx, md};
    block_reduce<4>(v, 0xCu);
    if (threadIdx.x == 0) {
        pu_out[0 * G + vb] = v[0];
        pu_out[1 * G + vb] = v[1];
        pu_out[2 * G + vb] = v[2];
        pu_out[3 * G + vb] = v[3];
    }
}

template <bool CHECON>
__global__ void __launch_bounds__(256)
k_pcg_update1(int ns, const PcgState *__restrict__ st, const double *__restrict__ ps, int Gs,
              double *__restrict__ pu_out, int G, double *__restrict__ x, double *__restrict__ r,
              double *__restrict__ d, const double *__restrict__ p, const double *__restrict__ u,
              const double *__restrict__ dinv)
{
    if (block_stopped(st)) return;
    const double pu = reduce_partials(ps, Gs, false);
    const double alpha = st->up / pu;
    update1_block<CHECON>(blockIdx.x, gridDim.x, ns, alpha, pu_out, G, x, r, d, p, u, dinv);
}

// update2: beta = (r.d)/up; p = d + p*beta (and its FP32 high and low
// parts into ps, shared-km contexts).  Reads st->up only.
__device__ __forceinline__ void update2_block(int vb, int nvb, int ns, double beta, const double *__restrict__ d,
                                              double *__restrict__ p, float2 *__restrict__ ps)
{
    for (int s = vb * blockDim.x + threadIdx.x; s < ns; s += nvb * blockDim.x) {
        const double pn = fma(p[s], beta, d[s]);
        p[s] = pn;
        if (ps) {
            float h, l;
            tc::split_f64(pn, h, l);
            ps[s] = make_float2(h, l);
        }
    }
}

__global__ void __launch_bounds__(256)
k_pcg_update2(int ns, const PcgState *__restrict__ st, const double *__restrict__ part, int G,
              const double *__restrict__ d, double *__restrict__ p, float2 *__restrict__ ps)
{
    if (block_stopped(st)) return;
    const double rd = reduce_partials(part, G, false);
    const double beta = rd / st->up;
    update2_block(blockIdx.x, gridDim.x, ns, beta, d, p, ps);
}

// finish (one block): the iteration's bookkeeping -- up for the next
// iteration, the iteration count and the stopping test (checon_par,
// maths.f90:1052-1062, or the relative residual).  It is the only kernel
// of an iteration that writes the state.
__global__ void __launch_bounds__(256)
k_pcg_finish(PcgState *__restrict__ st, const double *__restrict__ part, int G)
{
    if (block_stopped(st)) return;
    const double rd = reduce_partials(part, G, false);
    const double rr = reduce_partials(part + 1 * G, G, false);
    const bool checon = st->stop_mode == STOP_CHECON;   // uniform: written only by init kernels
    const double mx = checon ? reduce_partials(part + 2 * G, G, true) : 1.0;
    const double md = checon ? reduce_partials(part + 3 * G, G, true) : 0.0;
    if (threadIdx.x == 0) {
        const int k = st->iters + 1;
        const double metric = checon ? md / mx : sqrt(rr) / sqrt(st->ff);
        const bool conv = metric <= st->tol;
        st->up = rd;
        st->iters = k;
        st->rr = rr;
        st->metric = metric;
        st->converged = conv ? 1 : 0;
        if (!isfinite(rd) || !isfinite(mx)) st->err = 1;
        if (conv || k >= st->limit || st->err) st->stop = 1;
    }
}

// ---------------------------------------------------------------------------
// Persistent PCG iterations (p121.f90:90-104 with DOT_PRODUCT_P,
// maths.f90:168-215, and checon_par, maths.f90:1052-1062).  One cooperative
// launch runs the scatter, both update passes and the finish of an
// iteration -- and, in the FP64 form (ELEM64), the element products too and
// up to `niters` whole iterations -- with grid-wide barriers where the
// separate kernels have launch boundaries.  The launch has at most as many
// blocks as are resident at once.  Block b runs the virtual blocks b,
// b + gridDim.x, ... of the Gs-block scatter and of the G-block vector
// kernels through the same block bodies, and every block forms the
// reductions of the finish itself in the same fixed order, so the iterates
// and the stopping decisions are bitwise those of the separate kernels.
// Block 0 writes the state; the other blocks only read it at the start,
// before the first barrier.
struct PersistArgs {
    int nels, nn, ns, G, Gs, niters;
    const double *km64;   // FP64 storkm (ELEM64)
    const int *conn;
    void *ut;             // element results
    const int *node_ptr, *node_list;
    const uint8_t *fm;
    double *x, *r, *d, *p, *u;
    const double *dinv;
    double *part_s, *part_u;
    float2 *psplit;       // shared-km contexts: FP32 high/low parts of p
    PcgState *st;
    unsigned long long *bar;
    int *kerr;
};

template <typename UT, bool ELEM64, bool CHECON, int MINB, int PF>
__global__ void __launch_bounds__(256, MINB) k_pcg_persistent(PersistArgs a)
{
    if (block_stopped(a.st)) return;
    volatile PcgState *vs = a.st;
    double up = vs->up;
    int iters = vs->iters;
    const int limit = vs->limit;
    const double tol = vs->tol, ff = vs->ff;
    const int lane = threadIdx.x & 31;
    for (int it = 0; it < a.niters; ++it) {
        if (ELEM64) {
            const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
            const int nw = (gridDim.x * blockDim.x) >> 5;
            for (int e = warp; e < a.nels; e += nw)
                elem_warp<double, true>(e, lane, a.km64, a.conn, a.p, (double *)a.ut);
            if (!grid_barrier(a.bar, a.kerr, a.st)) return;
        }
        for (int vb = blockIdx.x; vb < a.Gs; vb += gridDim.x)
            scatter_block<UT, 0, !ELEM64, PF>(vb, a.Gs, a.nn, a.node_ptr, a.node_list, (const UT *)a.ut, a.fm, a.p,
                                          a.u, a.part_s);
        if (!grid_barrier(a.bar, a.kerr, a.st)) return;
        const double alpha = up / reduce_partials(a.part_s, a.Gs, false);
        for (int vb = blockIdx.x; vb < a.G; vb += gridDim.x)
            update1_block<CHECON>(vb, a.G, a.ns, alpha, a.part_u, a.G, a.x, a.r, a.d, a.p, a.u, a.dinv);
        if (!grid_barrier(a.bar, a.kerr, a.st)) return;
        const double rd = reduce_partials(a.part_u, a.G, false);
        const double beta = rd / up;
        for (int vb = blockIdx.x; vb < a.G; vb += gridDim.x) update2_block(vb, a.G, a.ns, beta, a.d, a.p, a.psplit);
        // the finish of k_pcg_finish, formed by every block
        const double rr = reduce_partials(a.part_u + a.G, a.G, false);
        const double mx = CHECON ? reduce_partials(a.part_u + 2 * a.G, a.G, true) : 1.0;
        const double md = CHECON ? reduce_partials(a.part_u + 3 * a.G, a.G, true) : 0.0;
        ++iters;
        const double metric = CHECON ? md / mx : sqrt(rr) / sqrt(ff);
        const bool conv = metric <= tol;
        const bool bad = !isfinite(rd) || !isfinite(mx);
        const bool stop = conv || iters >= limit || bad;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            vs->up = rd;
            vs->iters = iters;
            vs->rr = rr;
            vs->metric = metric;
            vs->converged = conv ? 1 : 0;
            if (bad) vs->err = 1;
            if (stop) vs->stop = 1;
        }
        up = rd;
        if (stop) return;
        if (it + 1 < a.niters && !grid_barrier(a.bar, a.kerr, a.st)) return;
    }
}

// Residual replacement (defect correction keeping the Krylov space): the
// recursive residual is replaced by the FP64 true residual rres = f - K x;
// d = diag*r and r.d are recomputed, the search direction p is kept.
__global__ void __launch_bounds__(256)
k_pcg_replace(int ns, const double *__restrict__ rres, const double *__restrict__ dinv,
              double *__restrict__ r, double *__restrict__ d, double *__restrict__ part, int G)
{
    double rd = 0.0, rr = 0.0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const double rv = rres[s];
        const double dv = dinv[s] * rv;
        r[s] = rv;
        d[s] = dv;
        rd = fma(rv, dv, rd);
        rr = fma(rv, rv, rr);
    }
    double v[2] = {rd, rr};
    block_reduce<2>(v, 0u);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = v[0];
        part[G + blockIdx.x] = v[1];
    }
}

__global__ void k_pcg_replace2(PcgState *st, const double *__restrict__ part, int G, double tol)
{
    const double rd = reduce_partials(part, G, false);
    const double rr = reduce_partials(part + G, G, false);
    if (threadIdx.x == 0) {
        st->up = rd;
        st->rr = rr;
        st->metric = sqrt(rr) / sqrt(st->ff);
        st->tol = tol;
        st->converged = 0;
        st->stop = (rr == 0.0) ? 1 : 0;
    }
}

__global__ void k_sum_partials(const double *__restrict__ part, int G, int nvals,
                               double *__restrict__ out)
{
    for (int k = 0; k < nvals; ++k) {
        const double v = reduce_partials(part + (size_t)k * G, G, false);
        if (threadIdx.x == 0) out[k] = v;
    }
}

__global__ void k_eq_to_slot(int ns, const int *__restrict__ slot_eq, const double *__restrict__ eq,
                             double *__restrict__ slot)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const int q = slot_eq[s];
        slot[s] = q > 0 ? eq[q - 1] : 0.0;
    }
}

__global__ void k_slot_to_eq(int neq, const int *__restrict__ eq_slot, const double *__restrict__ slot,
                             double *__restrict__ eq)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < neq; q += gridDim.x * blockDim.x)
        eq[q] = slot[eq_slot[q]];
}

__global__ void k_axpy(int ns, double *__restrict__ y, const double *__restrict__ x)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x)
        y[s] += x[s];
}

// Centroid stresses (p121.f90:112-123: nip=1 at the origin) of elements
// e0 .. e0+count-1, one thread per element; sig[6*k + c] for element e0+k.
// The shape-function derivatives at the centroid are the same for every
// element; the Jacobian, its inverse and the strains follow p121's order.
__global__ void __launch_bounds__(128)
k_centroid_stress(int e0, int count, const int *__restrict__ conn, const double *__restrict__ coord,
                  const double *__restrict__ me, const double *__restrict__ mv, int nmat,
                  const double *__restrict__ x, double *__restrict__ sig)
{
    __shared__ double der[60];
    if (threadIdx.x < 20) shape_der20(threadIdx.x, 0.0, 0.0, 0.0, &der[3 * threadIdx.x]);
    __syncthreads();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const int e = e0 + k;
        const double *co = coord + (size_t)e * 60;
        double jac[9];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                for (int m = 0; m < 20; ++m) s += der[a + 3 * m] * co[m + 20 * b];
                jac[a + 3 * b] = s;
            }
        det_invert3(jac);
        // eps = bee . eld (BEEMAT rows ex, ey, ez, gxy, gyz, gzx), deriv = jac^-1 der
        double eps[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int m = 0; m < 20; ++m) {
            const double d0 = der[3 * m], d1 = der[3 * m + 1], d2 = der[3 * m + 2];
            const double gx = jac[0] * d0 + jac[3] * d1 + jac[6] * d2;
            const double gy = jac[1] * d0 + jac[4] * d1 + jac[7] * d2;
            const double gz = jac[2] * d0 + jac[5] * d1 + jac[8] * d2;
            const int nd = conn[(size_t)e * 20 + m];
            const double ux = x[(size_t)3 * nd], uy = x[(size_t)3 * nd + 1], uz = x[(size_t)3 * nd + 2];
            eps[0] += gx * ux;
            eps[1] += gy * uy;
            eps[2] += gz * uz;
            eps[3] += gy * ux + gx * uy;
            eps[4] += gz * uy + gy * uz;
            eps[5] += gz * ux + gx * uz;
        }
        double d11, d12, d44;
        const int mi = nmat == 1 ? 0 : e;
        deemat3(me[mi], mv[mi], d11, d12, d44);
        double *o = sig + (size_t)6 * k;
        o[0] = d11 * eps[0] + d12 * eps[1] + d12 * eps[2];
        o[1] = d12 * eps[0] + d11 * eps[1] + d12 * eps[2];
        o[2] = d12 * eps[0] + d12 * eps[1] + d11 * eps[2];
        o[3] = d44 * eps[3];
        o[4] = d44 * eps[4];
        o[5] = d44 * eps[5];
    }
}

// Generic batched product of the xx3 layer (cuda_helpers.cu:144-177 semantics):
// one thread per row, FP64.
__global__ void k_matvec_rows(int n_mat, int n_row, int n_col, const double *__restrict__ lhs,
                              const double *__restrict__ mat, double *__restrict__ rhs)
{
    const size_t total = (size_t)n_mat * n_row;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total;
         g += (size_t)gridDim.x * blockDim.x) {
        const size_t m = g / n_row, i = g % n_row;
        const double *a = mat + m * n_row * (size_t)n_col + i;
        const double *x = lhs + m * n_col;
        double s = 0.0;
        for (int j = 0; j < n_col; ++j) s = fma(x[j], a[(size_t)j * n_row], s);
        rhs[g] = s;
    }
}

// Exercises the bounded mbarrier wait of the bulk-copy kernels on a barrier
// that nothing completes: one thread arms it for 16 bytes of transactions
// and issues no copy, so no copy is in flight when the wait gives up.  The
// kernel then records code 2 in the error word, as those kernels do.
__global__ void k_wait_probe(long long polls, int *err)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::mbar_fence_init();
        tc::mbar_expect_tx(&bar, 16);
        if (!tc::mbar_wait_n(&bar, 0, polls)) atomicExch(err, 2);
    }
}

// ---------------------------------------------------------------------------
// launchers
static int grid_for(const Ctx &c, long long work, int per_block, int max_per_sm)
{
    long long g = (work + per_block - 1) / per_block;
    const long long cap = (long long)c.nsm * max_per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

int launch_form_storkm(Ctx &c, int nip, bool exact_weights, bool keep32)
{
    double *gp = nullptr;
    if (cudaMallocAsync(&gp, sizeof(double) * 4 * 27, c.stream) != cudaSuccess) {
        set_error("form_storkm: cannot allocate the Gauss table");
        return 1;
    }
    k_sample<<<1, 1, 0, c.stream>>>(nip, exact_weights ? 1 : 0, gp);
    if (check_launch(c, "k_sample")) return 1;
    const int grid = c.nels < c.nsm * 16 ? c.nels : c.nsm * 16;
    if (c.kind == KIND_SOLID8)
        k_form_storkm<8><<<grid, kFormThreads, 0, c.stream>>>(c.nels, nip, gp, c.coord, c.mat_e, c.mat_v, c.nmat,
                                                              c.km64, nullptr, c.ediag);
    else
        k_form_storkm<20><<<grid, kFormThreads, 0, c.stream>>>(c.nels, nip, gp, c.coord, c.mat_e, c.mat_v, c.nmat,
                                                               c.km64, keep32 ? c.km32 : nullptr, c.ediag);
    if (check_launch(c, "k_form_storkm")) return 1;
    cudaFreeAsync(gp, c.stream);
    return 0;
}

int launch_sample(cudaStream_t stream, int nip, bool exact_weights, double *gp)
{
    k_sample<<<1, 1, 0, stream>>>(nip, exact_weights ? 1 : 0, gp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_sample: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int launch_form_storkm_raw(cudaStream_t stream, int nsm, int nels, int nip, const double *gp,
                           const double *coord, const double *me, const double *mv, int nmat, double *km64,
                           float *km32, double *ediag)
{
    const int grid = nels < nsm * 16 ? nels : nsm * 16;
    k_form_storkm<20><<<grid, kFormThreads, 0, stream>>>(nels, nip, gp, coord, me, mv, nmat, km64, km32, ediag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_form_storkm: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int launch_cast_km32(Ctx &c)
{
    const size_t n = (size_t)c.nels * 3600;
    k_cast_km32<<<c.nsm * 8, 256, 0, c.stream>>>(n, c.km64, c.km32);
    if (check_launch(c, "k_cast_km32")) return 1;
    k_extract_ediag<<<c.nsm * 8, 256, 0, c.stream>>>(c.nels, c.km64, c.ediag);
    return check_launch(c, "k_extract_ediag");
}

int launch_assemble_diag(Ctx &c)
{
    if (c.kind == KIND_SCALAR8) return launch_assemble_diag1(c);
    k_assemble_diag<<<grid_for(c, c.nn, 256, 8), 256, 0, c.stream>>>(
        c.nn, c.node_ptr, c.node_list, c.ediag, c.freemask, c.diag, c.dinv);
    return check_launch(c, "k_assemble_diag");
}

int launch_eq_to_slot(Ctx &c, const double *eq, double *slot)
{
    k_eq_to_slot<<<grid_for(c, c.nslots, 256, 8), 256, 0, c.stream>>>(c.nslots, c.slot_eq, eq, slot);
    return check_launch(c, "k_eq_to_slot");
}

int launch_slot_to_eq(Ctx &c, const double *slot, double *eq)
{
    k_slot_to_eq<<<grid_for(c, c.neq, 256, 8), 256, 0, c.stream>>>(c.neq, c.eq_slot, slot, eq);
    return check_launch(c, "k_slot_to_eq");
}

int launch_elem(Ctx &c, int prec, const double *p)
{
    if (c.kind == KIND_SCALAR8) return launch_elem8(c, p, c.st);
    if (c.kind == KIND_SOLID8) return launch_elem24(c, p, c.st);
    if (c.shared) return launch_elem_shared(c, prec, p, c.st);
    if (prec == PREC_FP32_SYM) return launch_elem_sym32(c, p, c.st);
    if (prec == PREC_FP16_SYM) return launch_elem_sym16(c, p, c.st);
    const int grid = grid_for(c, c.nels, 8, 8);
    if (prec == PREC_FP32_FULL) {
        k_elem<float, true><<<grid, 256, 0, c.stream>>>(c.nels, c.km32, c.conn, p, (float *)c.utemp, c.st);
    } else {
        k_elem<double, true><<<grid, 256, 0, c.stream>>>(c.nels, c.km64, c.conn, p, (double *)c.utemp, c.st);
    }
    return check_launch(c, "k_elem");
}

int launch_scatter(Ctx &c, int prec, int mode, const double *pf, double *out)
{
    if (c.kind == KIND_SCALAR8) return launch_scatter1(c, mode, pf, pf, out, mode == 0 ? c.st : nullptr);
    if (c.kind == KIND_SOLID8 && mode == 0) return launch_scatter3_fixed(c, pf, out, c.st);
    const PcgState *st = mode == 0 ? c.st : nullptr;
    if (prec != PREC_FP64) {
        if (mode == 0)
            k_scatter<float, 0><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const float *)c.utemp,
                                                            c.freemask, pf, out, c.part_s, st);
        else
            k_scatter<float, 1><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const float *)c.utemp,
                                                            c.freemask, pf, out, c.part_s, st);
    } else {
        if (mode == 0)
            k_scatter<double, 0><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const double *)c.utemp,
                                                             c.freemask, pf, out, c.part_s, st);
        else
            k_scatter<double, 1><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const double *)c.utemp,
                                                             c.freemask, pf, out, c.part_s, st);
    }
    return check_launch(c, "k_scatter");
}

// u = K p outside a PCG run (state-independent).
int launch_matvec(Ctx &c, int prec, const double *p, double *u)
{
    if (c.kind == KIND_SCALAR8) {
        if (launch_elem8(c, p, nullptr)) return 1;
        return launch_scatter1(c, 0, p, p, u, nullptr);
    }
    if (c.kind == KIND_SOLID8) {
        if (launch_elem24(c, p, nullptr)) return 1;
        return launch_scatter3_fixed(c, p, u, nullptr);
    }
    const int grid = grid_for(c, c.nels, 8, 8);
    if (c.shared) {
        if (launch_elem_shared(c, prec, p, nullptr)) return 1;
    } else if (prec == PREC_FP32_SYM) {
        if (launch_elem_sym32(c, p, nullptr)) return 1;
    } else if (prec == PREC_FP16_SYM) {
        if (launch_elem_sym16(c, p, nullptr)) return 1;
    } else {
        if (prec == PREC_FP32_FULL)
            k_elem<float, true><<<grid, 256, 0, c.stream>>>(c.nels, c.km32, c.conn, p, (float *)c.utemp, nullptr);
        else
            k_elem<double, true><<<grid, 256, 0, c.stream>>>(c.nels, c.km64, c.conn, p, (double *)c.utemp, nullptr);
        if (check_launch(c, "k_elem")) return 1;
    }
    if (prec != PREC_FP64)
        k_scatter<float, 0><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const float *)c.utemp,
                                                        c.freemask, p, u, c.part_s, nullptr);
    else
        k_scatter<double, 0><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const double *)c.utemp,
                                                         c.freemask, p, u, c.part_s, nullptr);
    return check_launch(c, "k_scatter");
}

// out += K x (FP64 storkm) at the free dofs: SCATTER accumulating into out
int launch_scatter_add64(Ctx &c, double *out)
{
    k_scatter<double, 2><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const double *)c.utemp,
                                                     c.freemask, nullptr, out, c.part_s, nullptr);
    return check_launch(c, "k_scatter");
}

int launch_residual(Ctx &c, const double *f, const double *x, double *rres)
{
    if (c.kind == KIND_SCALAR8) {
        if (launch_elem8(c, x, nullptr)) return 1;
        return launch_scatter1(c, 1, x, f, rres, nullptr);
    }
    const int grid = grid_for(c, c.nels, 8, 8);
    if (c.kind == KIND_SOLID8) {
        // f - K x with the plain K, as p122 forms r = loads - K x (p122.f90:142-146)
        if (launch_elem24(c, x, nullptr)) return 1;
    } else if (c.shared) {
        if (launch_elem_shared(c, PREC_FP64, x, nullptr)) return 1;
    } else {
        k_elem<double, true><<<grid, 256, 0, c.stream>>>(c.nels, c.km64, c.conn, x, (double *)c.utemp, nullptr);
        if (check_launch(c, "k_elem")) return 1;
    }
    k_scatter<double, 1><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const double *)c.utemp,
                                                     c.freemask, f, rres, c.part_s, nullptr);
    return check_launch(c, "k_scatter");
}

int launch_pcg_init(Ctx &c, const double *rhs, double *xsol, int stop_mode, double tol, int limit, bool keep_x)
{
    c.stop_mode = stop_mode;
    if (cudaMemsetAsync(c.gbar, 0, sizeof(unsigned long long) * kPersistSlots * kBarWords, c.stream) != cudaSuccess) {
        set_error("k_pcg_init: cannot reset the grid-barrier counters");
        return 1;
    }
    k_pcg_init<<<c.G, 256, 0, c.stream>>>(c.nslots, rhs, c.dinv, xsol, c.r, c.d, c.p, c.part_u, c.G, keep_x ? 1 : 0,
                                          c.shared ? c.psplit : nullptr);
    if (check_launch(c, "k_pcg_init")) return 1;
    k_pcg_init2<<<1, 256, 0, c.stream>>>(c.st, c.part_u, c.G, stop_mode, tol, limit);
    return check_launch(c, "k_pcg_init2");
}

int launch_update1(Ctx &c, double *xsol)
{
    if (c.stop_mode == STOP_CHECON)
        k_pcg_update1<true><<<c.G, 256, 0, c.stream>>>(c.nslots, c.st, c.part_s, c.Gs, c.part_u, c.G, xsol, c.r, c.d,
                                                       c.p, c.u, c.dinv);
    else
        k_pcg_update1<false><<<c.G, 256, 0, c.stream>>>(c.nslots, c.st, c.part_s, c.Gs, c.part_u, c.G, xsol, c.r, c.d,
                                                        c.p, c.u, c.dinv);
    return check_launch(c, "k_pcg_update1");
}

int launch_update2(Ctx &c)
{
    k_pcg_update2<<<c.G, 256, 0, c.stream>>>(c.nslots, c.st, c.part_u, c.G, c.d, c.p, c.shared ? c.psplit : nullptr);
    if (check_launch(c, "k_pcg_update2")) return 1;
    k_pcg_finish<<<1, 256, 0, c.stream>>>(c.st, c.part_u, c.G);
    return check_launch(c, "k_pcg_finish");
}

// Blocks of the cooperative launch of one persistent-kernel instantiation:
// at most the resident capacity, and no more than the virtual blocks (and,
// with the element phase, the element warps) give work.
template <typename UT, bool ELEM64, bool CHECON, int MINB, int PF>
static int persist_grid(const Ctx &c)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_persistent<UT, ELEM64, CHECON, MINB, PF>, 256,
                                                      0) != cudaSuccess ||
        per_sm < 1)
        return 0;
    long long want = c.G > c.Gs ? c.G : c.Gs;
    if (ELEM64) {
        const long long ew = ((long long)c.nels + 7) / 8;
        if (ew > want) want = ew;
    }
    const long long cap = (long long)per_sm * c.nsm;
    return (int)(want < cap ? want : cap);
}

template <typename UT, bool ELEM64, bool CHECON>
static int launch_persist_t(Ctx &c, double *xsol, int niters)
{
    constexpr int MINB = 4, PF = sizeof(UT) == 8 ? 4 : 8;
    const int idx = (ELEM64 ? 4 : 0) + (sizeof(UT) == 4 ? 2 : 0) + (CHECON ? 1 : 0);
    if (c.pk_grid[idx] == 0) c.pk_grid[idx] = persist_grid<UT, ELEM64, CHECON, MINB, PF>(c);
    const int grid = c.pk_grid[idx];
    if (grid < 1) {
        set_error("persistent PCG kernel: no resident block fits");
        return 1;
    }
    PersistArgs a;
    a.nels = c.nels; a.nn = c.nn; a.ns = c.nslots; a.G = c.G; a.Gs = c.Gs; a.niters = niters;
    a.km64 = c.km64; a.conn = c.conn; a.ut = c.utemp; a.node_ptr = c.node_ptr; a.node_list = c.node_list;
    a.fm = c.freemask; a.x = xsol; a.r = c.r; a.d = c.d; a.p = c.p; a.u = c.u; a.dinv = c.dinv;
    a.part_s = c.part_s; a.part_u = c.part_u; a.psplit = c.shared ? c.psplit : nullptr; a.st = c.st;
    a.bar = c.gbar + (size_t)idx * kBarWords; a.kerr = c.kerr;
    void *args[] = {&a};
    const cudaError_t e = cudaLaunchCooperativeKernel(
        (const void *)k_pcg_persistent<UT, ELEM64, CHECON, MINB, PF>, dim3(grid), dim3(256), args, 0, c.stream);
    c.launches++;
    if (e != cudaSuccess) {
        set_error("k_pcg_persistent: cooperative launch of %d blocks failed: %s", grid, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

bool persist_fused64(const Ctx &c, int prec)
{
    return c.persistent && prec == PREC_FP64 && !c.shared && c.kind == KIND_SOLID20;
}

int launch_pcg_tail(Ctx &c, int prec, double *xsol)
{
    const bool ck = c.stop_mode == STOP_CHECON;
    if (prec == PREC_FP64)
        return ck ? launch_persist_t<double, false, true>(c, xsol, 1) : launch_persist_t<double, false, false>(c, xsol, 1);
    return ck ? launch_persist_t<float, false, true>(c, xsol, 1) : launch_persist_t<float, false, false>(c, xsol, 1);
}

int launch_pcg_fused64(Ctx &c, double *xsol, int niters)
{
    return c.stop_mode == STOP_CHECON ? launch_persist_t<double, true, true>(c, xsol, niters)
                                      : launch_persist_t<double, true, false>(c, xsol, niters);
}

int launch_pcg_iteration(Ctx &c, int prec, double *xsol)
{
    if (c.persistent && c.kind == KIND_SOLID20) {
        if (persist_fused64(c, prec)) return launch_pcg_fused64(c, xsol, 1);
        if (launch_elem(c, prec, c.p)) return 1;
        return launch_pcg_tail(c, prec, xsol);
    }

    if (launch_elem(c, prec, c.p)) return 1;
    if (launch_scatter(c, prec, 0, c.p, c.u)) return 1;
    if (launch_update1(c, xsol)) return 1;
    return launch_update2(c);
}

int launch_wait_probe(Ctx &c, long long polls)
{
    k_wait_probe<<<1, 32, 0, c.stream>>>(polls, c.kerr);
    return check_launch(c, "k_wait_probe");
}

int launch_axpy(Ctx &c, double *y, const double *xv)
{
    k_axpy<<<grid_for(c, c.nslots, 256, 8), 256, 0, c.stream>>>(c.nslots, y, xv);
    return check_launch(c, "k_axpy");
}

int launch_replace(Ctx &c, double tol)
{
    k_pcg_replace<<<c.G, 256, 0, c.stream>>>(c.nslots, c.rres, c.dinv, c.r, c.d, c.part_r, c.G);
    if (check_launch(c, "k_pcg_replace")) return 1;
    k_pcg_replace2<<<1, 256, 0, c.stream>>>(c.st, c.part_r, c.G, tol);
    return check_launch(c, "k_pcg_replace2");
}

int launch_sum_partials(Ctx &c, int nvals, double *out_dev)
{
    k_sum_partials<<<1, 256, 0, c.stream>>>(c.part_s, c.Gs, nvals, out_dev);
    return check_launch(c, "k_sum_partials");
}

int launch_centroid_stress(Ctx &c, int e0, int count, const double *xslot, double *sig_dev)
{
    const int grid = grid_for(c, count, 128, 8);
    k_centroid_stress<<<grid, 128, 0, c.stream>>>(e0, count, c.conn, c.coord, c.mat_e, c.mat_v, c.nmat, xslot,
                                                  sig_dev);
    return check_launch(c, "k_centroid_stress");
}

int launch_matvec_generic(int n_mat, int n_row, int n_col, const double *lhs, const double *mat,
                          double *rhs, long long *launches)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm < 1) nsm = 1;
    if (n_row == 60 && n_col == 60) {
        long long g = ((long long)n_mat + 7) / 8;
        if (g > nsm * 8LL) g = nsm * 8LL;
        if (g < 1) g = 1;
        k_elem<double, false><<<(int)g, 256>>>(n_mat, mat, nullptr, lhs, rhs, nullptr);
    } else {
        long long g = ((long long)n_mat * n_row + 127) / 128;
        if (g > nsm * 16LL) g = nsm * 16LL;
        if (g < 1) g = 1;
        k_matvec_rows<<<(int)g, 128>>>(n_mat, n_row, n_col, lhs, mat, rhs);
    }
    if (launches) ++*launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("matrix_vector_multiplies: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

}  // namespace pf
