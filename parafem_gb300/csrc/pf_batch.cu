// pf_batch.cu -- continuous batching of many p121 solves on one GPU.
//
// Many meshes of different sizes live in shared device arenas at once.  One
// PCG iteration of every active solve is one launch per kernel:
//   * the element products walk the concatenated element ranges of the
//     active meshes (a warp finds its mesh by binary search in a segment
//     table);
//   * the scatter and the vector kernels run over per-mesh block ranges, so
//     every reduction (p.u, r.d, r.r, max|x|, max|dx|) is summed over the
//     blocks of ONE mesh in a fixed order.  A mesh's partition depends on its
//     own size only, so its result is bitwise the same alone and in any mix;
//   * a one-block-per-mesh finish kernel does each mesh's bookkeeping and
//     sets its stop flag; the next iterations skip stopped meshes.
// Requests are admitted while others iterate: their arrays are copied into
// free arena ranges and their storkm is formed on the same stream, between
// iterations of the running solves.  Converged solves retire at the next
// sync, which frees their ranges for waiting requests.  Admission is bounded
// by a device-memory budget fixed at creation (first-fit over the element
// and node arenas); a request that does not fit yet gets PF_BUSY.
//
// The solve is p121's Jacobi-PCG (p121.f90:86-104) stopped at
// ||r||_2/||f||_2 <= tol, with one of three element products chosen at
// creation: FP64 storkm, or the packed-symmetric FP32 (prec 32) or FP16
// (prec 16) storkm (products by the bulk-copy kernels of the single-mesh
// path, through a map from active element positions to arena elements) with
// FP64 residual replacement per mesh (the PF_MODE_MIXED / PF_MODE_MIXED16
// scheme: a mesh whose recursive residual has
// dropped 10x pauses, the host computes its FP64 true residual at the next
// sync and either retires it or replaces its residual and resumes it).
// Each retired solve reports the FP64 true residual ||f - K x||_2/||f||_2.
#include "pf_device.cuh"
#include "pfgpu.h"

#include <algorithm>
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <vector>

namespace pf {

namespace {

struct BSeg {
    int el0, nels;     // element range in the arena
    int node0, nn;     // node range (slots 3*node0 ...)
    int sid;           // state index
    int pbs, nbs;      // scatter blocks [pbs, pbs+nbs)
    int pbv, nbv;      // vector blocks  [pbv, pbv+nbv)
    long long el_cum;  // elements of the segments before this one
};

constexpr int kScatterNodes = 256;   // nodes per scatter block
constexpr int kVectorSlots = 2048;   // slots per vector block (8 per thread)

__device__ __forceinline__ void elem_product(size_t e, int lane, const double *__restrict__ km,
                                             const int *__restrict__ conn, const double *__restrict__ p,
                                             double *__restrict__ ut)
{
    const int j1 = lane + 32;
    const int nd = (lane < 20) ? conn[e * 20 + lane] : 0;
    const int n0 = __shfl_sync(FULLMASK, nd, lane / 3);
    const int n1 = __shfl_sync(FULLMASK, nd, j1 < 60 ? j1 / 3 : 0);
    const double p0 = p[(size_t)3 * n0 + lane % 3];
    const double p1 = (j1 < 60) ? p[(size_t)3 * n1 + j1 % 3] : 0.0;
    const double *ke = km + e * 3600 + 2 * lane;
    double a0 = 0.0, a1 = 0.0;
#pragma unroll 12
    for (int j = 0; j < 60; ++j) {
        const double pj = __shfl_sync(FULLMASK, j < 32 ? p0 : p1, j & 31);
        if (lane < 30) {
            const double2 k2 = __ldg(reinterpret_cast<const double2 *>(ke + 60 * j));
            a0 = fma(k2.x, pj, a0);
            a1 = fma(k2.y, pj, a1);
        }
    }
    if (lane < 30) {
        double2 o;
        o.x = a0;
        o.y = a1;
        reinterpret_cast<double2 *>(ut + e * 60)[lane] = o;
    }
}

// element products of every active mesh
__global__ void __launch_bounds__(256)
k_bt_elem(int nseg, const BSeg *__restrict__ segs, long long total, const double *__restrict__ km,
          const int *__restrict__ conn, const double *__restrict__ p, double *__restrict__ ut,
          const PcgState *__restrict__ st)
{
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long g = warp; g < total; g += nwarps) {
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (segs[mid].el_cum <= g) lo = mid;
            else hi = mid - 1;
        }
        const int sid = segs[lo].sid;
        if (st[sid].stop) continue;
        const size_t e = (size_t)segs[lo].el0 + (size_t)(g - segs[lo].el_cum);
        elem_product(e, lane, km, conn, p, ut);
    }
}

// arena element of every active element position (the segment table in
// element order), for the bulk-copy element kernel of the mixed engine
__global__ void k_bt_emap(int nseg, const BSeg *__restrict__ segs, long long total, int *__restrict__ emap)
{
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
         g += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (segs[mid].el_cum <= g) lo = mid;
            else hi = mid - 1;
        }
        emap[g] = segs[lo].el0 + (int)(g - segs[lo].el_cum);
    }
}

// residual replacement of one mesh: r = rres, d = dinv*r; partials r.d, r.r
__global__ void __launch_bounds__(256)
k_bt_replace1(BSeg S, const double *__restrict__ rres, const double *__restrict__ dinv, double *__restrict__ r,
              double *__restrict__ d, double *__restrict__ part, int cap)
{
    const size_t s0 = (size_t)3 * S.node0 + (size_t)blockIdx.x * kVectorSlots;
    const size_t s1 = min(s0 + kVectorSlots, (size_t)3 * (S.node0 + S.nn));
    double rd = 0.0, rr = 0.0;
    for (size_t s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
        const double rv = rres[s], dv = dinv[s] * rv;
        r[s] = rv;
        d[s] = dv;
        rd = fma(rv, dv, rd);
        rr = fma(rv, rv, rr);
    }
    double v[2] = {rd, rr};
    block_reduce<2>(v, 0u);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = v[0];
        part[cap + blockIdx.x] = v[1];
    }
}

__global__ void k_bt_replace2(BSeg S, const double *__restrict__ part, int cap, double thr,
                              PcgState *__restrict__ st)
{
    const double rd = reduce_partials(part, S.nbv, false);
    const double rr = reduce_partials(part + cap, S.nbv, false);
    if (threadIdx.x == 0) {
        PcgState &T = st[S.sid];
        T.up = rd;
        T.rr = rr;
        T.tol = thr;
        T.converged = 0;
        T.stop = rr == 0.0 ? 1 : 0;
    }
}

// element products of one mesh (residual at retirement)
__global__ void __launch_bounds__(256)
k_bt_elem1(BSeg S, const double *__restrict__ km, const int *__restrict__ conn, const double *__restrict__ p,
           double *__restrict__ ut)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int g = warp; g < S.nels; g += nwarps) elem_product((size_t)S.el0 + g, lane, km, conn, p, ut);
}

// node-centric scatter of one node (ascending element order).  list[]
// holds contribution indices e*20+a: FP64 results sit at ci*3, FP32 results
// are node-padded float4s at ci and are summed in FP32.
template <typename UT, int MODE>
__device__ __forceinline__ double scatter_node(int n, const int2 *__restrict__ nptr, const int *__restrict__ list,
                                               const UT *__restrict__ ut, const uint8_t *__restrict__ fm,
                                               const double *__restrict__ pf, double *__restrict__ out)
{
    const int2 pr = nptr[n];
    UT a0 = 0, a1 = 0, a2 = 0;
    for (int k = pr.x; k < pr.y; k += 8) {
        int ci[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) ci[i] = (k + i < pr.y) ? __ldg(list + k + i) : -1;
        if constexpr (sizeof(UT) == 4) {
            float4 v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (ci[i] >= 0) v[i] = __ldg(reinterpret_cast<const float4 *>(ut) + ci[i]);
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (ci[i] >= 0) {
                    a0 += v[i].x;
                    a1 += v[i].y;
                    a2 += v[i].z;
                }
        } else {
            double v[8][3];
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (ci[i] >= 0) {
                    const double *q = ut + (size_t)ci[i] * 3;
                    v[i][0] = q[0];
                    v[i][1] = q[1];
                    v[i][2] = q[2];
                }
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (ci[i] >= 0) {
                    a0 += v[i][0];
                    a1 += v[i][1];
                    a2 += v[i][2];
                }
        }
    }
    const int m = fm[n];
    const double a[3] = {(double)a0, (double)a1, (double)a2};
    double loc = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const size_t s = (size_t)3 * n + d;
        const bool fr = (m >> d) & 1;
        if (MODE == 0) {
            const double uv = fr ? a[d] : 0.0;
            out[s] = uv;
            loc = fma(pf[s], uv, loc);
        } else {
            const double rv = fr ? pf[s] - a[d] : 0.0;
            out[s] = rv;
            loc = fma(rv, rv, loc);
        }
    }
    return loc;
}

template <typename UT>
__global__ void __launch_bounds__(256)
k_bt_scatter(const int *__restrict__ blk, const BSeg *__restrict__ segs, const int2 *__restrict__ nptr,
             const int *__restrict__ list, const UT *__restrict__ ut, const uint8_t *__restrict__ fm,
             const double *__restrict__ p, double *__restrict__ u, double *__restrict__ part,
             const PcgState *__restrict__ st)
{
    const int b = blockIdx.x;
    const BSeg &S = segs[blk[b]];
    if (st[S.sid].stop) return;   // no kernel writes the flag meanwhile: uniform per block
    const int n = S.node0 + (b - S.pbs) * kScatterNodes + threadIdx.x;
    double v[1] = {n < S.node0 + S.nn ? scatter_node<UT, 0>(n, nptr, list, ut, fm, p, u) : 0.0};
    block_reduce<1>(v, 0u);
    if (threadIdx.x == 0) part[b] = v[0];
}

// residual rres = f - K x of one mesh; partials of rres.rres per local block
__global__ void __launch_bounds__(256)
k_bt_residual1(BSeg S, const int2 *__restrict__ nptr, const int *__restrict__ list,
               const double *__restrict__ ut, const uint8_t *__restrict__ fm, const double *__restrict__ f,
               double *__restrict__ rres, double *__restrict__ part)
{
    const int n = S.node0 + blockIdx.x * kScatterNodes + threadIdx.x;
    double v[1] = {n < S.node0 + S.nn ? scatter_node<double, 1>(n, nptr, list, ut, fm, f, rres) : 0.0};
    block_reduce<1>(v, 0u);
    if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// Jacobi diagonal of one mesh (ascending element order per node)
__global__ void k_bt_diag(BSeg S, const int2 *__restrict__ nptr, const int *__restrict__ list,
                          const double *__restrict__ ed, const uint8_t *__restrict__ fm,
                          double *__restrict__ dinv)
{
    const int n = S.node0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= S.node0 + S.nn) return;
    const int2 pr = nptr[n];
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int k = pr.x; k < pr.y; ++k) {
        const double *q = ed + (size_t)list[k] * 3;
        a0 += q[0];
        a1 += q[1];
        a2 += q[2];
    }
    const int m = fm[n];
    const double a[3] = {a0, a1, a2};
    for (int d = 0; d < 3; ++d) dinv[(size_t)3 * n + d] = ((m >> d) & 1) ? 1.0 / a[d] : 0.0;
}

// init of one mesh: x = 0, r = f, d = dinv*r, p = d; partials r.d, r.r
__global__ void __launch_bounds__(256)
k_bt_init1(BSeg S, const double *__restrict__ f, const double *__restrict__ dinv, double *__restrict__ x,
           double *__restrict__ r, double *__restrict__ d, double *__restrict__ p, double *__restrict__ part, int cap)
{
    const size_t s0 = (size_t)3 * S.node0 + (size_t)blockIdx.x * kVectorSlots;
    const size_t s1 = min(s0 + kVectorSlots, (size_t)3 * (S.node0 + S.nn));
    double rd = 0.0, rr = 0.0;
    for (size_t s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
        const double rv = f[s], dv = dinv[s] * rv;
        x[s] = 0.0;
        r[s] = rv;
        d[s] = dv;
        p[s] = dv;
        rd = fma(rv, dv, rd);
        rr = fma(rv, rv, rr);
    }
    double v[2] = {rd, rr};
    block_reduce<2>(v, 0u);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = v[0];
        part[cap + blockIdx.x] = v[1];
    }
}

__global__ void k_bt_init2(BSeg S, const double *__restrict__ part, int cap, PcgState *__restrict__ st)
{
    const double rd = reduce_partials(part, S.nbv, false);
    const double rr = reduce_partials(part + cap, S.nbv, false);
    if (threadIdx.x == 0) {
        PcgState &T = st[S.sid];
        T.up = rd;
        T.ff = rr;
        T.rr = rr;
        T.metric = 1.0;
        T.iters = 0;
        T.converged = rr == 0.0 ? 1 : 0;
        T.stop = rr == 0.0 ? 1 : 0;
        T.err = 0;
    }
}

// one block per active mesh: alpha = (r.d)/(p.u) from the scatter's partials,
// formed once per mesh (not once per vector block: the FP64 reduction of a
// large mesh's partials in every block costs more than the update itself)
__global__ void __launch_bounds__(256)
k_bt_alpha(const BSeg *__restrict__ segs, PcgState *__restrict__ st, const double *__restrict__ part_s)
{
    const BSeg &S = segs[blockIdx.x];
    if (st[S.sid].stop) return;
    const double pu = reduce_partials(part_s + S.pbs, S.nbs, false);
    if (threadIdx.x == 0) st[S.sid].alpha = st[S.sid].up / pu;
}

__global__ void __launch_bounds__(256)
k_bt_update1(const int *__restrict__ blk, const BSeg *__restrict__ segs, const PcgState *__restrict__ st,
             double *__restrict__ part_u, int capv, double *__restrict__ x, double *__restrict__ r,
             double *__restrict__ d, const double *__restrict__ p, const double *__restrict__ u,
             const double *__restrict__ dinv)
{
    const int b = blockIdx.x;
    const BSeg &S = segs[blk[b]];
    if (st[S.sid].stop) return;
    const double alpha = st[S.sid].alpha;
    const size_t s0 = (size_t)3 * S.node0 + (size_t)(b - S.pbv) * kVectorSlots;
    const size_t s1 = min(s0 + kVectorSlots, (size_t)3 * (S.node0 + S.nn));
    // batched solves stop on the relative residual, so checon_par's max|x|
    // and max|dx| (three FP64 operations per slot on GB300's slow FP64
    // unit) are not formed
    double rd = 0.0, rr = 0.0;
    for (size_t s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
        x[s] = fma(p[s], alpha, x[s]);
        const double rn = fma(-u[s], alpha, r[s]);
        r[s] = rn;
        const double dn = dinv[s] * rn;
        d[s] = dn;
        rd = fma(rn, dn, rd);
        rr = fma(rn, rn, rr);
    }
    double v[2] = {rd, rr};
    block_reduce<2>(v, 0u);
    if (threadIdx.x == 0) {
        part_u[0 * (size_t)capv + b] = v[0];
        part_u[1 * (size_t)capv + b] = v[1];
    }
}

__global__ void __launch_bounds__(256)
k_bt_update2(const int *__restrict__ blk, const BSeg *__restrict__ segs, const PcgState *__restrict__ st,
             const double *__restrict__ part_u, const double *__restrict__ d, double *__restrict__ p)
{
    const int b = blockIdx.x;
    const BSeg &S = segs[blk[b]];
    if (st[S.sid].stop) return;
    const double rd = reduce_partials(part_u + S.pbv, S.nbv, false);
    const double beta = rd / st[S.sid].up;
    const size_t s0 = (size_t)3 * S.node0 + (size_t)(b - S.pbv) * kVectorSlots;
    const size_t s1 = min(s0 + kVectorSlots, (size_t)3 * (S.node0 + S.nn));
    for (size_t s = s0 + threadIdx.x; s < s1; s += blockDim.x) p[s] = fma(p[s], beta, d[s]);
}

// one block per active mesh: the iteration's bookkeeping
__global__ void __launch_bounds__(256)
k_bt_finish(const BSeg *__restrict__ segs, PcgState *__restrict__ st, const double *__restrict__ part_u, int capv)
{
    const BSeg &S = segs[blockIdx.x];
    if (st[S.sid].stop) return;
    const double rd = reduce_partials(part_u + S.pbv, S.nbv, false);
    const double rr = reduce_partials(part_u + capv + S.pbv, S.nbv, false);
    if (threadIdx.x == 0) {
        PcgState &T = st[S.sid];
        const int k = T.iters + 1;
        const double metric = sqrt(rr) / sqrt(T.ff);   // batched solves: relative residual
        const bool conv = metric <= T.tol;
        T.up = rd;
        T.iters = k;
        T.rr = rr;
        T.metric = metric;
        T.converged = conv ? 1 : 0;
        if (!isfinite(rd) || !isfinite(rr)) T.err = 1;
        if (conv || k >= T.limit || T.err) T.stop = 1;
    }
}

__global__ void k_bt_sum(const double *__restrict__ part, int n, double *__restrict__ out)
{
    const double v = reduce_partials(part, n, false);
    if (threadIdx.x == 0) *out = v;
}

// ---------------------------------------------------------------------------
// first-fit allocator over [0, cap)
struct FreeList {
    std::map<long long, long long> free;   // start -> length
    void init(long long cap) { free.clear(); if (cap > 0) free[0] = cap; }
    long long take(long long n)
    {
        for (auto it = free.begin(); it != free.end(); ++it)
            if (it->second >= n) {
                const long long s = it->first, len = it->second;
                free.erase(it);
                if (len > n) free[s + n] = len - n;
                return s;
            }
        return -1;
    }
    void give(long long s, long long n)
    {
        auto it = free.emplace(s, n).first;
        auto nx = std::next(it);
        if (nx != free.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free.erase(nx);
        }
        if (it != free.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free.erase(it);
            }
        }
    }
};

struct Req {
    int id = 0, nels = 0, nn = 0, neq = 0, limit = 0;
    double tol = 0.0;
    int corrections = 0;
    int el0 = 0, node0 = 0, sid = 0;
    int nbs = 0, nbv = 0;
    std::vector<int> eq_slot;   // local slot of equation q+1
};

struct Done {
    int id, iters, neq;
    double relres;
    std::vector<double> x;
};

struct Batch {
    int device = 0, nsm = 1;
    int prec = 64;                   // 64: FP64 products; 32: FP32 products + FP64 residual replacement
    cudaStream_t stream = nullptr;
    int *kerr = nullptr;             // bulk-copy wait timeouts of the element kernel
    int *emap = nullptr;             // [cap_el] arena element of each active element (prec 32 and 16)
    long long cap_el = 0, cap_nodes = 0;
    int max_meshes = 0, capb_s = 0, capb_v = 0;
    // arenas
    double *km64 = nullptr, *coord = nullptr, *ediag = nullptr, *ut = nullptr, *mat_e = nullptr, *mat_v = nullptr;
    float *km32p = nullptr;          // packed-symmetric FP32 storkm (prec 32): 1832 floats per element
    uint32_t *km16p = nullptr;       // packed-symmetric FP16 storkm (prec 16): 916 words per element
    int *conn = nullptr, *list = nullptr;
    int2 *nptr = nullptr;
    uint8_t *fm = nullptr;
    double *f = nullptr, *x = nullptr, *r = nullptr, *d = nullptr, *p = nullptr, *u = nullptr, *dinv = nullptr,
           *rres = nullptr;
    double *part_s = nullptr, *part_u = nullptr, *part_i = nullptr, *scr = nullptr, *gp = nullptr;
    PcgState *st = nullptr, *hst = nullptr;
    BSeg *d_segs = nullptr;
    int *d_blk_s = nullptr, *d_blk_v = nullptr;
    // pinned staging
    unsigned char *stage = nullptr;
    size_t stage_bytes = 0;
    cudaEvent_t stage_ev = nullptr;
    int gp_nip = 0;
    // host bookkeeping
    FreeList el_free, node_free;
    std::vector<int> sid_free;
    std::map<int, Req> active;       // id -> request (in the tables once activated)
    std::vector<int> order;          // active ids in table order
    std::vector<int> pending;        // admitted, not yet in the tables
    bool dirty = false;
    int nseg = 0, nblk_s = 0, nblk_v = 0;
    long long total_el = 0;
    std::deque<Done> done;
    int next_id = 0;
    long long launches = 0;
    // CUDA graph of one pf_batch_launch chunk, re-captured when the tables
    // change (and updated in place when the topology allows)
    bool use_graphs = true;
    long long version = 0;           // bumped by every table rebuild
    cudaGraphExec_t g_exec = nullptr;
    int g_iters = 0;
    long long g_version = -1, g_launches = 0;
};

#define BCK(call)                                                                        \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return PF_FAILURE;                                                           \
        }                                                                                \
    } while (0)

int launched(Batch &B, const char *name)
{
    B.launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: launch failed: %s", name, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

Batch *get_batch(void **h)
{
    if (!h || !*h) {
        set_error("null batch handle");
        return nullptr;
    }
    Batch *B = (Batch *)*h;
    if (cudaSetDevice(B->device) != cudaSuccess) {
        set_error("cannot select device %d", B->device);
        return nullptr;
    }
    return B;
}

void free_batch(Batch &B)
{
    void *ptrs[] = {B.km32p, B.km16p, B.kerr, B.emap, B.km64, B.coord, B.ediag, B.ut, B.mat_e, B.mat_v, B.conn, B.list, B.nptr, B.fm, B.f, B.x, B.r,
                    B.d, B.p, B.u, B.dinv, B.rres, B.part_s, B.part_u, B.part_i, B.scr, B.gp, B.st, B.d_segs,
                    B.d_blk_s, B.d_blk_v};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (B.hst) cudaFreeHost(B.hst);
    if (B.stage) cudaFreeHost(B.stage);
    if (B.stage_ev) cudaEventDestroy(B.stage_ev);
    if (B.g_exec) cudaGraphExecDestroy(B.g_exec);
    if (B.stream) cudaStreamDestroy(B.stream);
}

// Rebuilds the segment and block tables from the active requests.
int rebuild_tables(Batch &B)
{
    for (int id : B.pending) B.order.push_back(id);
    B.pending.clear();
    std::vector<BSeg> segs;
    std::vector<int> bs, bv;
    long long cum = 0;
    for (int id : B.order) {
        Req &q = B.active[id];
        BSeg S;
        S.el0 = q.el0;
        S.nels = q.nels;
        S.node0 = q.node0;
        S.nn = q.nn;
        S.sid = q.sid;
        S.pbs = (int)bs.size();
        S.nbs = q.nbs;
        S.pbv = (int)bv.size();
        S.nbv = q.nbv;
        S.el_cum = cum;
        cum += q.nels;
        const int m = (int)segs.size();
        for (int i = 0; i < q.nbs; ++i) bs.push_back(m);
        for (int i = 0; i < q.nbv; ++i) bv.push_back(m);
        segs.push_back(S);
    }
    if ((int)bs.size() > B.capb_s || (int)bv.size() > B.capb_v) {
        set_error("batch block tables overflow");
        return 1;
    }
    B.nseg = (int)segs.size();
    B.nblk_s = (int)bs.size();
    B.nblk_v = (int)bv.size();
    B.total_el = cum;
    BCK(cudaStreamSynchronize(B.stream));
    if (B.nseg > 0) {
        BCK(cudaMemcpy(B.d_segs, segs.data(), segs.size() * sizeof(BSeg), cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(B.d_blk_s, bs.data(), bs.size() * sizeof(int), cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(B.d_blk_v, bv.data(), bv.size() * sizeof(int), cudaMemcpyHostToDevice));
        if (B.prec != 64) {
            long long g = (cum + 255) / 256;
            if (g > (long long)B.nsm * 8) g = (long long)B.nsm * 8;
            k_bt_emap<<<(int)g, 256, 0, B.stream>>>(B.nseg, B.d_segs, cum, B.emap);
            if (launched(B, "k_bt_emap")) return 1;
        }
    }
    B.dirty = false;
    ++B.version;
    return 0;
}

BSeg seg_of(const Req &q)
{
    BSeg S;
    S.el0 = q.el0;
    S.nels = q.nels;
    S.node0 = q.node0;
    S.nn = q.nn;
    S.sid = q.sid;
    S.pbs = 0;
    S.nbs = q.nbs;
    S.pbv = 0;
    S.nbv = q.nbv;
    S.el_cum = 0;
    return S;
}

// A paused mesh: FP64 true residual; retire it (results to the host) or, in
// the mixed mode while the true residual is above tol, replace its residual
// and let it run on.
int check_or_retire(Batch &B, int id)
{
    Req &q = B.active[id];
    const BSeg S = seg_of(q);
    const int ge = (q.nels + 7) / 8 < B.nsm * 8 ? (q.nels + 7) / 8 : B.nsm * 8;
    k_bt_elem1<<<ge, 256, 0, B.stream>>>(S, B.km64, B.conn, B.x, B.ut);
    if (launched(B, "k_bt_elem1")) return 1;
    k_bt_residual1<<<q.nbs, 256, 0, B.stream>>>(S, B.nptr, B.list, B.ut, B.fm, B.f, B.rres, B.part_i);
    if (launched(B, "k_bt_residual1")) return 1;
    k_bt_sum<<<1, 256, 0, B.stream>>>(B.part_i, q.nbs, B.scr);
    if (launched(B, "k_bt_sum")) return 1;
    double rr = 0.0;
    BCK(cudaMemcpyAsync(&rr, B.scr, sizeof(double), cudaMemcpyDeviceToHost, B.stream));
    BCK(cudaStreamSynchronize(B.stream));
    const PcgState &T = B.hst[q.sid];
    const double relt = T.ff > 0 ? std::sqrt(rr) / std::sqrt(T.ff) : 0.0;
    if (B.prec != 64 && relt > q.tol && T.iters < q.limit && !T.err) {
        const double thr = 0.1 * relt > q.tol ? 0.1 * relt : 0.5 * q.tol;
        k_bt_replace1<<<q.nbv, 256, 0, B.stream>>>(S, B.rres, B.dinv, B.r, B.d, B.part_i, B.capb_v);
        if (launched(B, "k_bt_replace1")) return 1;
        k_bt_replace2<<<1, 256, 0, B.stream>>>(S, B.part_i, B.capb_v, thr, B.st);
        if (launched(B, "k_bt_replace2")) return 1;
        ++q.corrections;
        return 0;
    }
    const size_t ns = (size_t)3 * q.nn;
    std::vector<double> xs(ns);
    BCK(cudaMemcpyAsync(xs.data(), B.x + (size_t)3 * q.node0, ns * sizeof(double), cudaMemcpyDeviceToHost,
                        B.stream));
    BCK(cudaStreamSynchronize(B.stream));
    Done dn;
    dn.id = id;
    dn.iters = T.iters;
    dn.neq = q.neq;
    dn.relres = T.err ? NAN : relt;
    dn.x.resize(q.neq);
    for (int e = 0; e < q.neq; ++e) dn.x[e] = xs[q.eq_slot[e]];
    B.done.push_back(std::move(dn));
    B.el_free.give(q.el0, q.nels);
    B.node_free.give(q.node0, q.nn);
    B.sid_free.push_back(q.sid);
    B.order.erase(std::find(B.order.begin(), B.order.end(), id));
    B.active.erase(id);
    B.dirty = true;
    return 0;
}

// n batched PCG iterations over every active mesh, launched on B.stream.
int batch_iterations(Batch &B, int n)
{
    long long ge = (B.total_el + 7) / 8;
    if (ge > (long long)B.nsm * 8) ge = (long long)B.nsm * 8;
    if (ge < 1) ge = 1;
    for (int i = 0; i < n; ++i) {
        if (B.prec == 16) {
            if (launch_elem_sym16_mapped(B.stream, B.nsm, (int)B.total_el, B.km16p, B.conn, B.p, (float *)B.ut,
                                         B.kerr, B.emap))
                return 1;
            B.launches++;
            k_bt_scatter<float><<<B.nblk_s, 256, 0, B.stream>>>(B.d_blk_s, B.d_segs, B.nptr, B.list,
                                                                (const float *)B.ut, B.fm, B.p, B.u, B.part_s,
                                                                B.st);
        } else if (B.prec == 32) {
            if (launch_elem_sym32_mapped(B.stream, B.nsm, (int)B.total_el, B.km32p, B.conn, B.p, (float *)B.ut,
                                         B.kerr, B.emap))
                return 1;
            B.launches++;
            k_bt_scatter<float><<<B.nblk_s, 256, 0, B.stream>>>(B.d_blk_s, B.d_segs, B.nptr, B.list,
                                                                (const float *)B.ut, B.fm, B.p, B.u, B.part_s,
                                                                B.st);
        } else {
            k_bt_elem<<<(int)ge, 256, 0, B.stream>>>(B.nseg, B.d_segs, B.total_el, B.km64, B.conn, B.p, B.ut,
                                                     B.st);
            if (launched(B, "k_bt_elem")) return 1;
            k_bt_scatter<double><<<B.nblk_s, 256, 0, B.stream>>>(B.d_blk_s, B.d_segs, B.nptr, B.list, B.ut, B.fm,
                                                                 B.p, B.u, B.part_s, B.st);
        }
        if (launched(B, "k_bt_scatter")) return 1;
        k_bt_alpha<<<B.nseg, 256, 0, B.stream>>>(B.d_segs, B.st, B.part_s);
        if (launched(B, "k_bt_alpha")) return 1;
        k_bt_update1<<<B.nblk_v, 256, 0, B.stream>>>(B.d_blk_v, B.d_segs, B.st, B.part_u, B.capb_v, B.x, B.r, B.d,
                                                      B.p, B.u, B.dinv);
        if (launched(B, "k_bt_update1")) return 1;
        k_bt_update2<<<B.nblk_v, 256, 0, B.stream>>>(B.d_blk_v, B.d_segs, B.st, B.part_u, B.d, B.p);
        if (launched(B, "k_bt_update2")) return 1;
        k_bt_finish<<<B.nseg, 256, 0, B.stream>>>(B.d_segs, B.st, B.part_u, B.capb_v);
        if (launched(B, "k_bt_finish")) return 1;
    }
    return 0;
}

// The graph of n iterations for the current tables: captured, then either
// patched into the existing executable graph or instantiated.
int batch_graph(Batch &B, int n)
{
    if (B.g_exec && B.g_iters == n && B.g_version == B.version) return 0;
    const long long l0 = B.launches;
    if (cudaStreamBeginCapture(B.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        set_error("batch graph: cannot begin capture");
        return 1;
    }
    const int bad = batch_iterations(B, n);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(B.stream, &g);
    B.g_launches = B.launches - l0;
    B.launches = l0;
    if (bad || ec != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        if (!bad) set_error("batch graph: capture failed: %s", cudaGetErrorString(ec));
        return 1;
    }
    if (B.g_exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(B.g_exec, g, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(B.g_exec);
            B.g_exec = nullptr;
        }
    }
    if (!B.g_exec) {
        const cudaError_t ei = cudaGraphInstantiate(&B.g_exec, g, 0);
        if (ei != cudaSuccess) {
            B.g_exec = nullptr;
            cudaGraphDestroy(g);
            set_error("batch graph: instantiate failed: %s", cudaGetErrorString(ei));
            return 1;
        }
    }
    cudaGraphDestroy(g);
    B.g_iters = n;
    B.g_version = B.version;
    return 0;
}

}  // namespace
}  // namespace pf

using namespace pf;

// ===========================================================================
extern "C" int pf_batch_create(const int *device, const long long *budget_bytes, const int *max_meshes,
                               const int *prec, void **batch)
try {
    if (!device || !budget_bytes || !max_meshes || !prec || !batch || *max_meshes < 1 ||
        *budget_bytes < (1LL << 20) || (*prec != 64 && *prec != 32 && *prec != 16)) {
        set_error("pf_batch_create: invalid arguments (prec must be 64, 32 or 16)");
        return PF_FAILURE;
    }
    *batch = nullptr;
    BCK(cudaSetDevice(*device));
    Batch *B = new (std::nothrow) Batch();
    if (!B) {
        set_error("pf_batch_create: out of host memory");
        return PF_FAILURE;
    }
    B->device = *device;
    B->prec = *prec;
    cudaDeviceGetAttribute(&B->nsm, cudaDevAttrMultiProcessorCount, B->device);
    if (B->nsm < 1) B->nsm = 1;
    B->max_meshes = *max_meshes;
    // bytes per element slot: storkm 28800 (+ packed FP32 7328 or FP16 3664
    // and the element map 4 for prec 32 / 16), coord 480, conn 80, element
    // diag 480, results 480, node list 80, material 16; nodes: 7 per element
    // slot at 8 (ptr) + 1 (mask) + 8 vectors x 24 bytes
    const long long per_el = 28800 + (B->prec == 32 ? 7328 + 4 : B->prec == 16 ? 3664 + 4 : 0) + 480 + 80 + 480 +
                             480 + 80 + 16 +
                             7 * (8 + 1 + 8 * 24);
    B->cap_el = *budget_bytes / per_el;
    if (B->cap_el > 0x7fffffffLL / 60) B->cap_el = 0x7fffffffLL / 60;
    B->cap_nodes = 7 * B->cap_el;
    B->capb_s = (int)(B->cap_nodes / kScatterNodes + B->max_meshes + 1);
    B->capb_v = (int)(3 * B->cap_nodes / kVectorSlots + B->max_meshes + 1);
    const size_t E = (size_t)B->cap_el, N = (size_t)B->cap_nodes;
    bool ok = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) == cudaSuccess;
    auto al = [&](void **ptr, size_t bytes) {
        if (ok && cudaMalloc(ptr, bytes ? bytes : 1) != cudaSuccess) ok = false;
    };
    al((void **)&B->km64, E * 3600 * 8);
    if (B->prec == 16) al((void **)&B->km16p, E * 916 * 4);
    if (B->prec == 32) al((void **)&B->km32p, E * 1832 * 4);
    if (B->prec != 64) al((void **)&B->emap, E * 4);
    al((void **)&B->kerr, 4);
    al((void **)&B->coord, E * 60 * 8);
    al((void **)&B->ediag, E * 60 * 8);
    al((void **)&B->ut, E * 60 * 8);
    al((void **)&B->mat_e, E * 8);
    al((void **)&B->mat_v, E * 8);
    al((void **)&B->conn, E * 20 * 4);
    al((void **)&B->list, E * 20 * 4);
    al((void **)&B->nptr, N * sizeof(int2));
    al((void **)&B->fm, N);
    double **vecs[] = {&B->f, &B->x, &B->r, &B->d, &B->p, &B->u, &B->dinv, &B->rres};
    for (double **v : vecs) al((void **)v, N * 3 * 8);
    al((void **)&B->part_s, (size_t)B->capb_s * 8);
    al((void **)&B->part_u, (size_t)2 * B->capb_v * 8);   // r.d and r.r partials
    al((void **)&B->part_i, (size_t)2 * B->capb_v * 8);
    al((void **)&B->scr, 64);
    al((void **)&B->gp, 27 * 4 * 8);
    al((void **)&B->st, (size_t)B->max_meshes * sizeof(PcgState));
    al((void **)&B->d_segs, (size_t)B->max_meshes * sizeof(BSeg));
    al((void **)&B->d_blk_s, (size_t)B->capb_s * 4);
    al((void **)&B->d_blk_v, (size_t)B->capb_v * 4);
    if (ok && cudaMallocHost((void **)&B->hst, (size_t)B->max_meshes * sizeof(PcgState)) != cudaSuccess) ok = false;
    if (ok && cudaEventCreateWithFlags(&B->stage_ev, cudaEventDisableTiming) != cudaSuccess) ok = false;
    if (!ok) {
        set_error("pf_batch_create: cannot allocate the arenas for a %lld-byte budget", *budget_bytes);
        free_batch(*B);
        delete B;
        return PF_FAILURE;
    }
    cudaMemset(B->st, 0, (size_t)B->max_meshes * sizeof(PcgState));
    cudaMemset(B->kerr, 0, sizeof(int));
    memset(B->hst, 0, (size_t)B->max_meshes * sizeof(PcgState));
    if ((B->prec == 32 && sym32_prepare()) || (B->prec == 16 && sym16_prepare())) {
        free_batch(*B);
        delete B;
        return PF_FAILURE;
    }
    B->el_free.init(B->cap_el);
    B->node_free.init(B->cap_nodes);
    for (int i = B->max_meshes - 1; i >= 0; --i) B->sid_free.push_back(i);
    *batch = B;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_batch_create");
}

extern "C" int pf_batch_destroy(void **batch)
try {
    if (!batch || !*batch) return PF_SUCCESS;
    Batch *B = (Batch *)*batch;
    cudaSetDevice(B->device);
    cudaStreamSynchronize(B->stream);
    free_batch(*B);
    delete B;
    *batch = nullptr;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_batch_destroy");
}

extern "C" int pf_batch_capacity(void **batch, long long *elements, long long *nodes)
try {
    Batch *B = get_batch(batch);
    if (!B || !elements || !nodes) return PF_FAILURE;
    *elements = B->cap_el;
    *nodes = B->cap_nodes;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_batch_capacity");
}

extern "C" int pf_batch_admit(void **batch, const int *nels_p, const int *nn_p, const int *neq_p, const int *g_num,
                              const int *g_g, const double *g_coord, const int *nmat_p, const double *e,
                              const double *v, const int *nip_p, const double *rhs, const double *tol,
                              const int *limit, int *id_out)
try {
    Batch *Bp = get_batch(batch);
    if (!Bp) return PF_FAILURE;
    Batch &B = *Bp;
    if (!nels_p || !nn_p || !neq_p || !g_num || !g_g || !g_coord || !nmat_p || !e || !v || !nip_p || !rhs ||
        !tol || !limit || !id_out) {
        set_error("pf_batch_admit: null argument");
        return PF_FAILURE;
    }
    const int nels = *nels_p, nn = *nn_p, neq = *neq_p, nmat = *nmat_p, nip = *nip_p;
    if (nels < 1 || nn < 1 || neq < 1 || (nmat != 1 && nmat != nels) || (nip != 8 && nip != 27) || *limit < 1) {
        set_error("pf_batch_admit: invalid sizes (nels=%d nn=%d neq=%d nmat=%d nip=%d)", nels, nn, neq, nmat, nip);
        return PF_FAILURE;
    }
    if (nels > B.cap_el || nn > B.cap_nodes) {
        set_error("pf_batch_admit: a %d-element mesh exceeds the batch capacity (%lld elements)", nels, B.cap_el);
        return PF_FAILURE;
    }
    // mesh tables in local numbering (validated before anything is reserved)
    std::vector<int> slot_eq(3 * (size_t)nn, -1), eq_slot(neq, -1), cnt(nn + 1, 0);
    for (size_t el = 0; el < (size_t)nels; ++el)
        for (int a = 0; a < 20; ++a) {
            const int nd = g_num[el * 20 + a];
            if (nd < 1 || nd > nn) {
                set_error("pf_batch_admit: g_num(%d,%zu)=%d outside 1..%d", a + 1, el + 1, nd, nn);
                return PF_FAILURE;
            }
            cnt[nd]++;
            for (int d = 0; d < 3; ++d) {
                const int q = g_g[el * 60 + 3 * a + d];
                if (q < 0 || q > neq) {
                    set_error("pf_batch_admit: g_g entry %d outside 0..%d", q, neq);
                    return PF_FAILURE;
                }
                int &se = slot_eq[3 * (size_t)(nd - 1) + d];
                if (se < 0) se = q;
                else if (se != q) {
                    set_error("pf_batch_admit: node %d dof %d has two equation numbers", nd, d + 1);
                    return PF_FAILURE;
                }
            }
        }
    for (size_t s = 0; s < slot_eq.size(); ++s) {
        const int q = slot_eq[s] < 0 ? 0 : slot_eq[s];
        if (q > 0) {
            if (eq_slot[q - 1] >= 0) {
                set_error("pf_batch_admit: equation %d belongs to two dofs", q);
                return PF_FAILURE;
            }
            eq_slot[q - 1] = (int)s;
        }
    }
    for (int q = 0; q < neq; ++q)
        if (eq_slot[q] < 0) {
            set_error("pf_batch_admit: equation %d is used by no element", q + 1);
            return PF_FAILURE;
        }
    // reserve: a state, an element range, a node range
    if (B.sid_free.empty()) return 2;   // PF_BUSY
    const long long el0 = B.el_free.take(nels);
    if (el0 < 0) return 2;
    const long long node0 = B.node_free.take(nn);
    if (node0 < 0) {
        B.el_free.give(el0, nels);
        return 2;
    }
    const int sid = B.sid_free.back();
    B.sid_free.pop_back();

    // staging (pinned), reused once the previous admission's copies are done
    const size_t b_coord = (size_t)nels * 60 * 8, b_conn = (size_t)nels * 20 * 4, b_list = b_conn;
    const size_t b_nptr = (size_t)nn * sizeof(int2), b_fm = ((size_t)nn + 7) / 8 * 8,
                 b_f = (size_t)nn * 3 * 8, b_mat = (size_t)nmat * 8;
    const size_t need = b_coord + b_conn + b_list + b_nptr + b_fm + b_f + 2 * b_mat + 64;
    BCK(cudaEventSynchronize(B.stage_ev));
    if (need > B.stage_bytes) {
        if (B.stage) cudaFreeHost(B.stage);
        B.stage = nullptr;
        B.stage_bytes = 0;
        BCK(cudaMallocHost((void **)&B.stage, need));
        B.stage_bytes = need;
    }
    unsigned char *w = B.stage;
    double *h_coord = (double *)w; w += b_coord;
    int *h_conn = (int *)w; w += b_conn;
    int *h_list = (int *)w; w += b_list;
    int2 *h_nptr = (int2 *)w; w += b_nptr;
    uint8_t *h_fm = (uint8_t *)w; w += b_fm;
    double *h_f = (double *)w; w += b_f;
    double *h_me = (double *)w; w += b_mat;
    double *h_mv = (double *)w;
    memcpy(h_coord, g_coord, b_coord);
    for (size_t k = 0; k < (size_t)nels * 20; ++k) h_conn[k] = (int)node0 + g_num[k] - 1;
    std::vector<int> beg(nn + 1, 0);
    for (int n = 0; n < nn; ++n) beg[n + 1] = beg[n] + cnt[n + 1];
    std::vector<int> fill(beg.begin(), beg.end() - 1);
    const int lbase = 20 * (int)el0;
    for (size_t el = 0; el < (size_t)nels; ++el)
        for (int a = 0; a < 20; ++a) {
            const int n = g_num[el * 20 + a] - 1;
            h_list[fill[n]++] = (int)((el0 + el) * 20 + a);   // local position, global contribution index
        }
    for (int n = 0; n < nn; ++n) {
        h_nptr[n].x = lbase + beg[n];
        h_nptr[n].y = lbase + beg[n + 1];
        uint8_t m = 0;
        for (int d = 0; d < 3; ++d)
            if (slot_eq[3 * (size_t)n + d] > 0) m |= (uint8_t)(1u << d);
        h_fm[n] = m;
        for (int d = 0; d < 3; ++d) {
            const int q = slot_eq[3 * (size_t)n + d];
            h_f[3 * (size_t)n + d] = q > 0 ? rhs[q - 1] : 0.0;
        }
    }
    memcpy(h_me, e, b_mat);
    memcpy(h_mv, v, b_mat);
    BCK(cudaMemcpyAsync(B.coord + (size_t)el0 * 60, h_coord, b_coord, cudaMemcpyHostToDevice, B.stream));
    BCK(cudaMemcpyAsync(B.conn + (size_t)el0 * 20, h_conn, b_conn, cudaMemcpyHostToDevice, B.stream));
    BCK(cudaMemcpyAsync(B.list + (size_t)el0 * 20, h_list, b_list, cudaMemcpyHostToDevice, B.stream));
    BCK(cudaMemcpyAsync(B.nptr + node0, h_nptr, b_nptr, cudaMemcpyHostToDevice, B.stream));
    BCK(cudaMemcpyAsync(B.fm + node0, h_fm, (size_t)nn, cudaMemcpyHostToDevice, B.stream));
    BCK(cudaMemcpyAsync(B.f + (size_t)3 * node0, h_f, b_f, cudaMemcpyHostToDevice, B.stream));
    BCK(cudaMemcpyAsync(B.mat_e + el0, h_me, b_mat, cudaMemcpyHostToDevice, B.stream));
    BCK(cudaMemcpyAsync(B.mat_v + el0, h_mv, b_mat, cudaMemcpyHostToDevice, B.stream));
    // state: tolerance, limit, stopping test
    PcgState T;
    memset(&T, 0, sizeof T);
    T.tol = B.prec != 64 ? (0.1 > *tol ? 0.1 : *tol) : *tol;   // mixed: first replacement threshold
    T.limit = *limit;
    T.stop_mode = STOP_RELRES;
    T.stop = 1;   // inactive until the init kernel runs
    B.hst[sid] = T;
    BCK(cudaMemcpyAsync(B.st + sid, &B.hst[sid], sizeof(PcgState), cudaMemcpyHostToDevice, B.stream));
    BCK(cudaEventRecord(B.stage_ev, B.stream));

    Req q;
    q.id = B.next_id++;
    q.nels = nels;
    q.nn = nn;
    q.neq = neq;
    q.el0 = (int)el0;
    q.node0 = (int)node0;
    q.sid = sid;
    q.nbs = (nn + kScatterNodes - 1) / kScatterNodes;
    q.nbv = (int)((3LL * nn + kVectorSlots - 1) / kVectorSlots);
    q.eq_slot = std::move(eq_slot);
    q.tol = *tol;
    q.limit = *limit;
    const BSeg S = seg_of(q);
    // storkm, diagonal, PCG start of this mesh
    if (B.gp_nip != nip) {
        if (launch_sample(B.stream, nip, false, B.gp)) return PF_FAILURE;
        B.gp_nip = nip;
    }
    if (launch_form_storkm_raw(B.stream, B.nsm, nels, nip, B.gp, B.coord + (size_t)el0 * 60, B.mat_e + el0,
                               B.mat_v + el0, nmat, B.km64 + (size_t)el0 * 3600, nullptr,
                               B.ediag + (size_t)el0 * 60))
        return PF_FAILURE;
    B.launches++;
    if (B.km32p) {
        if (launch_pack_sym32_raw(B.stream, B.nsm, nels, B.km64 + (size_t)el0 * 3600, B.km32p + (size_t)el0 * 1832))
            return PF_FAILURE;
        B.launches++;
    }
    if (B.km16p) {
        if (launch_pack_sym16_raw(B.stream, B.nsm, nels, B.km64 + (size_t)el0 * 3600, B.km16p + (size_t)el0 * 916))
            return PF_FAILURE;
        B.launches++;
    }
    k_bt_diag<<<(nn + 255) / 256, 256, 0, B.stream>>>(S, B.nptr, B.list, B.ediag, B.fm, B.dinv);
    if (launched(B, "k_bt_diag")) return PF_FAILURE;
    k_bt_init1<<<q.nbv, 256, 0, B.stream>>>(S, B.f, B.dinv, B.x, B.r, B.d, B.p, B.part_i, B.capb_v);
    if (launched(B, "k_bt_init1")) return PF_FAILURE;
    k_bt_init2<<<1, 256, 0, B.stream>>>(S, B.part_i, B.capb_v, B.st);
    if (launched(B, "k_bt_init2")) return PF_FAILURE;
    B.active[q.id] = std::move(q);
    B.pending.push_back(B.next_id - 1);
    B.dirty = true;
    *id_out = B.next_id - 1;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_batch_admit");
}

extern "C" int pf_batch_launch(void **batch, const int *iters)
try {
    Batch *Bp = get_batch(batch);
    if (!Bp || !iters || *iters < 1) {
        if (Bp) set_error("pf_batch_launch: iters must be >= 1");
        return PF_FAILURE;
    }
    Batch &B = *Bp;
    if (B.dirty && rebuild_tables(B)) return PF_FAILURE;
    if (B.nseg == 0) return PF_SUCCESS;
    if (!B.use_graphs) return batch_iterations(B, *iters) ? PF_FAILURE : PF_SUCCESS;
    if (batch_graph(B, *iters)) return PF_FAILURE;
    BCK(cudaGraphLaunch(B.g_exec, B.stream));
    B.launches += B.g_launches;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_batch_launch");
}

extern "C" int pf_batch_sync(void **batch, int *n_active, int *n_done)
try {
    Batch *Bp = get_batch(batch);
    if (!Bp) return PF_FAILURE;
    Batch &B = *Bp;
    BCK(cudaMemcpyAsync(B.hst, B.st, (size_t)B.max_meshes * sizeof(PcgState), cudaMemcpyDeviceToHost, B.stream));
    int kerr = 0;
    BCK(cudaMemcpyAsync(&kerr, B.kerr, sizeof(int), cudaMemcpyDeviceToHost, B.stream));
    BCK(cudaStreamSynchronize(B.stream));
    if (kerr) {
        cudaMemsetAsync(B.kerr, 0, sizeof(int), B.stream);
        set_error("pf_batch_sync: a shared-memory bulk-copy wait of the element kernel timed out");
        return PF_FAILURE;
    }
    std::vector<int> fin;
    for (int id : B.order)
        if (B.hst[B.active[id].sid].stop) fin.push_back(id);
    for (int id : fin)
        if (check_or_retire(B, id)) return PF_FAILURE;
    if (n_active) *n_active = (int)(B.order.size() + B.pending.size());
    if (n_done) *n_done = (int)B.done.size();
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_batch_sync");
}

extern "C" int pf_batch_collect(void **batch, int *id, int *iters, double *relres, double *x, const int *x_cap,
                                int *neq)
try {
    Batch *Bp = get_batch(batch);
    if (!Bp || !id || !iters || !relres || !neq) return PF_FAILURE;
    Batch &B = *Bp;
    if (B.done.empty()) {
        set_error("pf_batch_collect: no finished solve");
        return PF_FAILURE;
    }
    Done &dn = B.done.front();
    *neq = dn.neq;
    if (x) {
        if (!x_cap || *x_cap < dn.neq) {
            set_error("pf_batch_collect: x holds %d values, the solve has %d", x_cap ? *x_cap : 0, dn.neq);
            return PF_FAILURE;
        }
        memcpy(x, dn.x.data(), (size_t)dn.neq * sizeof(double));
    }
    *id = dn.id;
    *iters = dn.iters;
    *relres = dn.relres;
    B.done.pop_front();
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_batch_collect");
}

extern "C" int pf_batch_set_graphs(void **batch, const int *on)
try {
    Batch *B = get_batch(batch);
    if (!B || !on) return PF_FAILURE;
    B->use_graphs = *on != 0;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_batch_set_graphs");
}

extern "C" int pf_batch_launches(void **batch, long long *count)
try {
    Batch *B = get_batch(batch);
    if (!B || !count) return PF_FAILURE;
    *count = B->launches;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_batch_launches");
}
