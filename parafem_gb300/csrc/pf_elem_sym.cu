// pf_elem_sym.cu -- element products from packed-symmetric FP32 storkm,
// staged through shared memory by the bulk-copy (TMA) engine.
//
// storkm(60,60,e) is symmetric (B'DB), so the inner PCG of the mixed solver
// keeps only its upper triangle: U(i,j), i <= j, column-major,
// offset T(j)+i with T(j) = j(j+1)/2 -- 1,830 floats, padded to 1,832
// (7,328 bytes, a multiple of 16) per element.  That halves the dominant
// HBM stream of an iteration (the idea of xx16's packed DSPMV storage,
// src/programs/dev/xx16/xx16.f90:393-459).
//
// Kernel structure (one persistent CTA of 14 warps per SM):
//   * every warp owns a ring of NSTAGE shared-memory stages with one
//     mbarrier each; lane 0 issues cp.async.bulk of the next elements'
//     packed blocks into the ring (complete_tx on the stage's mbarrier);
//   * the warp gathers p for the element two positions ahead in registers,
//     so the global gather overlaps the current element's arithmetic;
//   * lanes 0..29 own rows l and 59-l and walk the 60 columns, reading
//     U(min(i,j), max(i,j)) from shared memory (at most 2-way bank conflicts)
//     with p(j) broadcast from a per-warp slot.  Each row is summed in
//     ascending column order with FMA, as the full-storage kernel does.
// Every wait on an mbarrier is bounded; a wait that runs out writes 2 to
// the context's device error word and the warp drains its in-flight copies
// (again with a bound) before it returns.
#include "pf_internal.h"
#include "pf_tc.cuh"

#include <cstdint>

namespace pf {

using namespace tc;

namespace {

constexpr int kPacked = 1832;                 // floats per element (1830 + 2 pad)
constexpr int kPackedBytes = kPacked * 4;     // 7328
constexpr unsigned kFull = 0xffffffffu;
}  // namespace

// Packs the upper triangle of the FP64 storkm into FP32 (one warp per element).
__global__ void k_pack_sym32(int nels, const double *__restrict__ km, float *__restrict__ kp)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int e = warp; e < nels; e += nwarps) {
        const double *ke = km + (size_t)e * 3600;
        float *out = kp + (size_t)e * kPacked;
        for (int j = 0; j < 60; ++j)
            for (int i = lane; i <= j; i += 32) out[j * (j + 1) / 2 + i] = (float)ke[60 * j + i];
        if (lane < 2) out[1830 + lane] = 0.0f;
    }
}

// u_e = K_e p_e for every element, K_e from the packed FP32 triangle.
// kWarps warps per CTA, kStages shared-memory stages per warp (tuned at
// run time among the instantiations below).
template <int kWarps, int kStages>
__global__ void __launch_bounds__(kWarps * 32, 1)
k_elem_sym32(int nels, const float *__restrict__ kp, const int *__restrict__ conn,
             const double *__restrict__ p, float *__restrict__ ut, const PcgState *__restrict__ st,
             int *__restrict__ err, const int *__restrict__ emap)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    float *stage = reinterpret_cast<float *>(smem) + (size_t)w * kStages * kPacked;
    float *pslot = reinterpret_cast<float *>(smem + (size_t)kWarps * kStages * kPackedBytes) + w * 64;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + (size_t)kWarps * kStages * kPackedBytes +
                                                 kWarps * 64 * 4) + w * kStages;
    static_assert((kWarps * kStages * kPackedBytes + kWarps * 64 * 4) % 8 == 0, "mbarrier alignment");

    // stop flag: uniform per warp (no block barrier after this point)
    int stopped = 0;
    if (lane == 0 && st) stopped = st->stop;
    stopped = __shfl_sync(kFull, stopped, 0);
    if (stopped) return;

    // this CTA's contiguous element range, warps interleaved inside it
    const int per_cta = (nels + gridDim.x - 1) / gridDim.x;
    const int e0 = blockIdx.x * per_cta;
    const int e1 = min(nels, e0 + per_cta);
    const int first = e0 + w;
    if (first >= e1) return;
    const int nmine = (e1 - first + kWarps - 1) / kWarps;   // elements of this warp
    // the k-th element of this warp; emap (serving batches) maps the
    // position among the active elements to the arena element
    auto elem = [&](int k) { const int g = first + k * kWarps; return emap ? __ldg(emap + g) : g; };

    if (lane == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (lane == 0) {
        for (int s = 0; s < kStages && s < nmine; ++s) {
            mbar_expect_tx(&bar[s], kPackedBytes);
            bulk_g2s(stage + s * kPacked, kp + (size_t)elem(s) * kPacked, kPackedBytes, &bar[s]);
        }
    }

    // gather pipeline: p values of element k (two floats per lane: dofs lane,
    // lane+32) and the connectivity of element k+1
    const int j1 = lane + 32;
    auto gather = [&](int e, int nd, float &a, float &b) {
        const int n0 = __shfl_sync(kFull, nd, lane / 3);
        const int n1 = __shfl_sync(kFull, nd, j1 < 60 ? j1 / 3 : 0);
        a = (float)p[(size_t)3 * n0 + lane % 3];
        b = j1 < 60 ? (float)p[(size_t)3 * n1 + j1 % 3] : 0.0f;
    };
    int conn_next = 0;
    float pa = 0.f, pb = 0.f;
    {
        const int nd0 = lane < 20 ? conn[(size_t)elem(0) * 20 + lane] : 0;
        gather(elem(0), nd0, pa, pb);
        if (nmine > 1 && lane < 20) conn_next = conn[(size_t)elem(1) * 20 + lane];
    }

    // rows owned by this lane and the running offsets of U(min,max) in column j
    const int ra = lane, rb = 59 - lane;
    const bool active = lane < 30;
    bool failed = false;
    int k = 0;
    for (; k < nmine; ++k) {
        const int s = k % kStages;
        const uint32_t parity = (uint32_t)((k / kStages) & 1);
        // prefetch: p of element k+1, connectivity of element k+2
        float na = 0.f, nb = 0.f;
        if (k + 1 < nmine) gather(elem(k + 1), conn_next, na, nb);
        int conn_next2 = 0;
        if (k + 2 < nmine && lane < 20) conn_next2 = conn[(size_t)elem(k + 2) * 20 + lane];

        // p of element k into the warp's slot
        pslot[lane] = pa;
        if (j1 < 60) pslot[j1] = pb;
        const bool ok = __all_sync(kFull, mbar_wait(&bar[s], parity));
        if (!ok) {
            failed = true;
            break;
        }
        __syncwarp();
        const float *U = stage + s * kPacked;
        float acc_a = 0.f, acc_b = 0.f;
        if (active) {
            int ia = ra * (ra + 1) / 2;   // U(min(ra,0), max(ra,0)) = T(ra) + 0
            int ib = rb * (rb + 1) / 2;
#pragma unroll 4
            for (int j = 0; j < 60; ++j) {
                const float pj = pslot[j];
                acc_a = fmaf(U[ia], pj, acc_a);
                acc_b = fmaf(U[ib], pj, acc_b);
                ia += (j < ra) ? 1 : j + 1;   // T(ra)+j -> T(ra)+j+1, then T(j)+ra -> T(j+1)+ra
                ib += (j < rb) ? 1 : j + 1;
            }
            float *o = ut + (size_t)elem(k) * 80;   // node-padded: row i at (i/3)*4 + i%3
            o[(ra / 3) * 4 + ra % 3] = acc_a;
            o[(rb / 3) * 4 + rb % 3] = acc_b;
        }
        __syncwarp();   // every lane is done with stage s and the p slot
        if (lane == 0 && k + kStages < nmine) {
            fence_proxy_async();
            mbar_expect_tx(&bar[s], kPackedBytes);
            bulk_g2s(stage + s * kPacked, kp + (size_t)elem(k + kStages) * kPacked, kPackedBytes, &bar[s]);
        }
        pa = na;
        pb = nb;
        conn_next = conn_next2;
    }
    if (failed) {
        if (lane == 0) atomicExch(err, 2);
        // drain: wait (bounded) for every copy this warp still has in flight
        for (int kk = k; kk < nmine && kk < k + kStages; ++kk)
            mbar_wait(&bar[kk % kStages], (uint32_t)((kk / kStages) & 1));
    }
}

template <int W, int S>
constexpr size_t sym_smem_bytes()
{
    return (size_t)W * S * kPackedBytes + W * 64 * 4 + W * S * 8;
}

template <int W, int S>
static int launch_sym_cfg(Ctx &c, const double *p, const PcgState *st)
{
    constexpr size_t smem = sym_smem_bytes<W, S>();
    static_assert(smem <= 227 * 1024, "shared memory per CTA");
    cudaError_t e;
    // the attribute is set once per context and configuration, before any
    // stream capture (the autotuner launches every configuration first)
    const unsigned long long bit = 1ull << (W * 4 + S);   // W <= 15, S <= 3
    if (!(c.sym_attr & bit)) {
        e = cudaFuncSetAttribute(k_elem_sym32<W, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            set_error("k_elem_sym32: cannot reserve %zu bytes of shared memory: %s", smem, cudaGetErrorString(e));
            return 1;
        }
        c.sym_attr |= bit;
    }
    const int grid = c.nels < c.nsm * W ? (c.nels + W - 1) / W : c.nsm;
    k_elem_sym32<W, S><<<grid, W * 32, smem, c.stream>>>(c.nels, c.km32p, c.conn, p, (float *)c.utemp, st, c.kerr,
                                                         nullptr);
    c.launches++;
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_elem_sym32: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

// the tuned configurations: (warps per CTA, stages per warp)
static const int kSymCfg[][2] = {{14, 2}, {12, 2}, {8, 3}};
constexpr int kNumSymCfg = 3;

static int launch_sym_index(Ctx &c, int idx, const double *p, const PcgState *st)
{
    switch (idx) {
    case 1: return launch_sym_cfg<12, 2>(c, p, st);
    case 2: return launch_sym_cfg<8, 3>(c, p, st);
    default: return launch_sym_cfg<14, 2>(c, p, st);
    }
}

// The serving engine's entry points: the (14, 2) configuration over n
// active elements mapped to arena elements by emap.  sym32_prepare sets the
// shared-memory attribute; call it once per device before any stream capture.
int sym32_prepare()
{
    constexpr size_t smem = sym_smem_bytes<14, 2>();
    const cudaError_t e = cudaFuncSetAttribute(k_elem_sym32<14, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
    if (e != cudaSuccess) {
        set_error("k_elem_sym32: cannot reserve %zu bytes of shared memory: %s", smem, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int launch_elem_sym32_mapped(cudaStream_t stream, int nsm, int n, const float *kp, const int *conn, const double *p,
                             float *ut, int *err, const int *emap)
{
    if (n <= 0) return 0;
    constexpr int W = 14;
    const int grid = n < nsm * W ? (n + W - 1) / W : nsm;
    k_elem_sym32<W, 2><<<grid, W * 32, sym_smem_bytes<W, 2>(), stream>>>(n, kp, conn, p, ut, nullptr, err, emap);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_elem_sym32: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int launch_pack_sym32_raw(cudaStream_t stream, int nsm, int nels, const double *km, float *kp)
{
    k_pack_sym32<<<nsm * 8, 256, 0, stream>>>(nels, km, kp);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_pack_sym32: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int launch_pack_sym32(Ctx &c)
{
    k_pack_sym32<<<c.nsm * 8, 256, 0, c.stream>>>(c.nels, c.km64, c.km32p);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_pack_sym32: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int launch_elem_sym32(Ctx &c, const double *p, const PcgState *st)
{
    return launch_sym_index(c, c.sym_cfg, p, st);
}

// Autotuner: times every configuration on this mesh (one warm-up and three
// timed launches each, CUDA events on the context stream) and keeps the
// fastest in c.sym_cfg.
int autotune_sym32(Ctx &c, const double *p)
{
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        set_error("autotune: cannot create events");
        return 1;
    }
    float best = 1e30f;
    int best_i = 0;
    for (int i = 0; i < kNumSymCfg; ++i) {
        if (launch_sym_index(c, i, p, nullptr)) return 1;
        cudaEventRecord(a, c.stream);
        for (int r = 0; r < 3; ++r)
            if (launch_sym_index(c, i, p, nullptr)) return 1;
        cudaEventRecord(b, c.stream);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        c.tune_ms[i] = ms / 3.0f;
        if (ms < best) {
            best = ms;
            best_i = i;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    set_sym_config(c, best_i);
    return 0;
}

void set_sym_config(Ctx &c, int idx)
{
    c.sym_cfg = idx;
    c.sym_warps = kSymCfg[idx][0];
    c.sym_stages = kSymCfg[idx][1];
}

}  // namespace pf
