// pf_scalar8.cu -- p123's path: 3-D Laplace (potential flow) with 8-node
// bricks and one freedom per node, solved by the same element-by-element
// Jacobi-PCG (src/programs/5th_ed/p123/p123.f90).
//
// A context set up with pf_setup_scalar8 holds 8-node connectivity, one slot
// per node, and storkc(8,8,e).  The PCG vector kernels are the 20-node path's
// (they work on slots); this file adds:
//   k_form_storkc     kc = sum_gp (kx dx dx' + ky dy dy' + kz dz dz') det w
//                     (p123.f90:70-85), eight threads per element;
//   k_elem8           u_e = kc_e p_e, eight threads per element (thread i
//                     owns row i and reads column j of kc_e as the group's
//                     contiguous 64 bytes), FP64 in ascending column order;
//   k_scatter1        node-centric sum in ascending element order, with
//                     p123's fixed freedoms: u = p * store at a node fixed by
//                     the penalty method (p123.f90:127-131);
//   k_assemble_diag1  the Jacobi diagonal (p123.f90:87-94).
#include "pf_device.cuh"

namespace pf {

// Eight threads per element; thread c owns column c of kcx, kcy, kcz.
__global__ void __launch_bounds__(128)
k_form_storkc(int nels, int nip, const double *__restrict__ gp, const double *__restrict__ coord, double kx,
              double ky, double kz, double *__restrict__ kc, double *__restrict__ ediag)
{
    const int c = threadIdx.x & 7;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)nels * 8;
         t += (long long)gridDim.x * blockDim.x) {
        const size_t e = (size_t)(t >> 3);
        const double *co = coord + e * 24;   // coord(8,3)
        double kxx[8], kyy[8], kzz[8];
        for (int r = 0; r < 8; ++r) kxx[r] = kyy[r] = kzz[r] = 0.0;
        for (int g = 0; g < nip; ++g) {
            const double xi = gp[4 * g], eta = gp[4 * g + 1], zeta = gp[4 * g + 2], w = gp[4 * g + 3];
            double der[24];
            for (int l = 0; l < 8; ++l) shape_der8(l, xi, eta, zeta, &der[3 * l]);
            double jac[9];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double s = 0.0;
                    for (int k = 0; k < 8; ++k) s += der[a + 3 * k] * co[k + 8 * b];
                    jac[a + 3 * b] = s;
                }
            const double det = det_invert3(jac);
            double dv[24];
            for (int l = 0; l < 8; ++l)
                for (int a = 0; a < 3; ++a)
                    dv[a + 3 * l] = jac[a] * der[3 * l] + jac[a + 3] * der[3 * l + 1] + jac[a + 6] * der[3 * l + 2];
            for (int r = 0; r < 8; ++r) {
                kxx[r] += dv[3 * r] * dv[3 * c] * det * w;
                kyy[r] += dv[3 * r + 1] * dv[3 * c + 1] * det * w;
                kzz[r] += dv[3 * r + 2] * dv[3 * c + 2] * det * w;
            }
        }
        double *out = kc + e * 64 + 8 * c;
        for (int r = 0; r < 8; ++r) out[r] = kxx[r] * kx + kyy[r] * ky + kzz[r] * kz;
        ediag[e * 8 + c] = out[c];
    }
}

// u_e = kc_e p_e: eight threads per element, thread i owns row i
__global__ void __launch_bounds__(256)
k_elem8(int nels, const double *__restrict__ kc, const int *__restrict__ conn, const double *__restrict__ p,
        double *__restrict__ ut, const PcgState *__restrict__ st)
{
    if (block_stopped(st)) return;
    const int i = threadIdx.x & 7;
    const unsigned gmask = 0xFFu << (threadIdx.x & 24);   // the 8 lanes of this element
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)nels * 8;
         t += (long long)gridDim.x * blockDim.x) {
        const size_t e = (size_t)(t >> 3);
        const double pi = p[conn[e * 8 + i]];
        const double *k = kc + e * 64 + i;
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < 8; ++j) acc = fma(k[8 * j], __shfl_sync(gmask, pi, (threadIdx.x & 24) + j), acc);
        ut[e * 8 + i] = acc;
    }
}

// Node-centric scatter (one freedom per node).  list[] holds e*8+a.
//   MODE 0: out = u, partial p.u          (pf = p)
//   MODE 1: out = f - u, partial out.out  (pf = f)
// A fixed node (fstore != 0) takes u = p * store (p123.f90:127-131);
// a restrained node gets 0.
template <int MODE>
__global__ void __launch_bounds__(256)
k_scatter1(int nn, const int *__restrict__ ptr, const int *__restrict__ list, const double *__restrict__ ut,
           const uint8_t *__restrict__ fm, const double *__restrict__ fstore, const double *__restrict__ xin,
           const double *__restrict__ pf, double *__restrict__ out, double *__restrict__ part,
           const PcgState *__restrict__ st)
{
    if (block_stopped(st)) return;
    double loc = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += gridDim.x * blockDim.x) {
        double a = 0.0;
        for (int k = ptr[n]; k < ptr[n + 1]; ++k) a += ut[list[k]];
        const bool fr = fm[n] & 1;
        const double fs = fstore[n];
        if (fs != 0.0) a = xin[n] * fs;
        if (MODE == 0) {
            const double uv = fr ? a : 0.0;
            out[n] = uv;
            loc = fma(pf[n], uv, loc);
        } else {
            const double rv = fr ? pf[n] - a : 0.0;
            out[n] = rv;
            loc = fma(rv, rv, loc);
        }
    }
    double v[1] = {loc};
    block_reduce<1>(v, 0u);
    if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

__global__ void k_assemble_diag1(int nn, const int *__restrict__ ptr, const int *__restrict__ list,
                                 const double *__restrict__ ed, const uint8_t *__restrict__ fm,
                                 double *__restrict__ diag, double *__restrict__ dinv, double *__restrict__ fstore)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += gridDim.x * blockDim.x) {
        double a = 0.0;
        for (int k = ptr[n]; k < ptr[n + 1]; ++k) a += ed[list[k]];
        const bool fr = fm[n] & 1;
        diag[n] = fr ? a : 0.0;
        dinv[n] = fr ? 1.0 / a : 0.0;
        fstore[n] = 0.0;
    }
}

// fixed freedoms (p123.f90:104-110): diag += penalty, store = diag
__global__ void k_set_fixed(int nfix, const int *__restrict__ slots, double penalty, double *__restrict__ diag,
                            double *__restrict__ dinv, double *__restrict__ fstore)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nfix; i += gridDim.x * blockDim.x) {
        const int s = slots[i];
        const double d = diag[s] + penalty;
        diag[s] = d;
        dinv[s] = 1.0 / d;
        fstore[s] = d;
    }
}

static int launched8(Ctx &c, const char *name)
{
    c.launches++;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: launch failed: %s", name, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

static int grid8(const Ctx &c, long long work, int per_block, int max_per_sm)
{
    long long g = (work + per_block - 1) / per_block;
    if (g > (long long)c.nsm * max_per_sm) g = (long long)c.nsm * max_per_sm;
    return (int)(g < 1 ? 1 : g);
}

int launch_form_storkc(Ctx &c, int nip, double kx, double ky, double kz)
{
    double *gp = nullptr;
    if (cudaMallocAsync(&gp, sizeof(double) * 4 * 27, c.stream) != cudaSuccess) {
        set_error("form_storkc: cannot allocate the Gauss table");
        return 1;
    }
    if (launch_sample(c.stream, nip, false, gp)) return 1;
    c.launches++;
    k_form_storkc<<<grid8(c, (long long)c.nels * 8, 128, 16), 128, 0, c.stream>>>(c.nels, nip, gp, c.coord, kx, ky,
                                                                                   kz, c.km64, c.ediag);
    if (launched8(c, "k_form_storkc")) return 1;
    cudaFreeAsync(gp, c.stream);
    return 0;
}

int launch_elem8(Ctx &c, const double *p, const PcgState *st)
{
    k_elem8<<<grid8(c, (long long)c.nels * 8, 256, 8), 256, 0, c.stream>>>(c.nels, c.km64, c.conn, p,
                                                                           (double *)c.utemp, st);
    return launched8(c, "k_elem8");
}

int launch_scatter1(Ctx &c, int mode, const double *xin, const double *pf, double *out, const PcgState *st)
{
    if (mode == 0)
        k_scatter1<0><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const double *)c.utemp, c.freemask,
                                                  c.fstore, xin, pf, out, c.part_s, st);
    else
        k_scatter1<1><<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const double *)c.utemp, c.freemask,
                                                  c.fstore, xin, pf, out, c.part_s, st);
    return launched8(c, "k_scatter1");
}

int launch_assemble_diag1(Ctx &c)
{
    k_assemble_diag1<<<grid8(c, c.nn, 256, 8), 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, c.ediag,
                                                                    c.freemask, c.diag, c.dinv, c.fstore);
    return launched8(c, "k_assemble_diag1");
}

int launch_set_fixed(Ctx &c, int nfix, const int *slots_dev, double penalty)
{
    k_set_fixed<<<grid8(c, nfix, 256, 4), 256, 0, c.stream>>>(nfix, slots_dev, penalty, c.diag, c.dinv, c.fstore);
    return launched8(c, "k_set_fixed");
}

}  // namespace pf
