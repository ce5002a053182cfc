// pf_solid8.cu -- 8-node elasticity bricks (three freedoms per node, 24 per
// element), the elements of p122's demo deck (src/programs/5th_ed/p122/p122.f90
// with nod = 8).  A context set up with pf_setup_solid8 keeps the 20-node
// path's slots (three per node), node-centric scatter and PCG vector kernels;
// storkm(24,24,e) is formed by k_form_storkm<8> (pf_kernels.cu).  This file
// adds the FP64 element product and the product scatter with fixed freedoms:
//   k_elem24        u_e = storkm_e p_e, one warp per element: lane i < 24 owns
//                   row i, p_e is gathered once per lane and broadcast by
//                   shuffles, FMA in ascending column order (as the serial
//                   MATMUL);
//   k_scatter3_fix  the node-centric sum of the 20-node path (ascending
//                   element order per node) with p122's fixed freedoms: at a
//                   freedom fixed by the penalty method the product is
//                   p * store * fscale (p122.f90:153-158: p * store on the
//                   first plastic iteration, 0 after), and the partial p.u
//                   uses that value.
#include "pf_device.cuh"

namespace pf {

__global__ void __launch_bounds__(256)
k_elem24(int nels, const double *__restrict__ km, const int *__restrict__ conn, const double *__restrict__ p,
         double *__restrict__ ut, const PcgState *__restrict__ st)
{
    if (st && st->stop) return;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int row = lane < 24 ? lane : 23;
    for (int e = warp; e < nels; e += nwarps) {
        const int node = conn[(size_t)e * 8 + row / 3];
        const double pv = p[(size_t)3 * node + row % 3];
        const double *k = km + (size_t)e * 576 + row;   // column j of storkm_e at k[24 j]
        double acc = 0.0;
#pragma unroll 8
        for (int j = 0; j < 24; ++j) acc = fma(k[24 * j], __shfl_sync(FULLMASK, pv, j), acc);
        if (lane < 24) ut[(size_t)e * 24 + lane] = acc;
    }
}

// out = u at free freedoms (restrained 0; fixed: p * store * fscale),
// partial p.u per block
__global__ void __launch_bounds__(256)
k_scatter3_fix(int nn, const int *__restrict__ ptr, const int *__restrict__ list, const double *__restrict__ ut,
               const uint8_t *__restrict__ fm, const double *__restrict__ fstore, const double *__restrict__ fscale,
               const double *__restrict__ p, double *__restrict__ out, double *__restrict__ part,
               const PcgState *__restrict__ st)
{
    if (block_stopped(st)) return;
    const double fsc = *fscale;
    double loc = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += gridDim.x * blockDim.x) {
        double a[3] = {0.0, 0.0, 0.0};
        for (int k = ptr[n]; k < ptr[n + 1]; ++k) {
            const double *q = ut + (size_t)list[k] * 3;
            a[0] += q[0];
            a[1] += q[1];
            a[2] += q[2];
        }
        const int m = fm[n];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const size_t s = (size_t)3 * n + d;
            const double fs = fstore[s];
            double uv = (m >> d) & 1 ? a[d] : 0.0;
            if (fs != 0.0) uv = p[s] * fs * fsc;
            out[s] = uv;
            loc = fma(p[s], uv, loc);
        }
    }
    double v[1] = {loc};
    block_reduce<1>(v, 0u);
    if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

static int launched24(Ctx &c, const char *name)
{
    c.launches++;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: launch failed: %s", name, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int launch_elem24(Ctx &c, const double *p, const PcgState *st)
{
    long long g = ((long long)c.nels + 7) / 8;
    if (g > (long long)c.nsm * 8) g = (long long)c.nsm * 8;
    k_elem24<<<(int)(g < 1 ? 1 : g), 256, 0, c.stream>>>(c.nels, c.km64, c.conn, p, (double *)c.utemp, st);
    return launched24(c, "k_elem24");
}

int launch_scatter3_fixed(Ctx &c, const double *p, double *out, const PcgState *st)
{
    k_scatter3_fix<<<c.Gs, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, (const double *)c.utemp, c.freemask,
                                               c.fstore, c.fscale, p, out, c.part_s, st);
    return launched24(c, "k_scatter3_fix");
}

}  // namespace pf
