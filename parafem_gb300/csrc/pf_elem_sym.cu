// pf_elem_sym.cu -- element products from packed-symmetric FP32 storkm,
// staged through shared memory by the bulk-copy (TMA) engine.
//
// storkm(60,60,e) is symmetric (B'DB), so the inner PCG of the mixed solver
// keeps each entry once, in FP32: 1,830 floats, padded to 1,832 (7,328
// bytes, a multiple of 16) per element.  That halves the dominant HBM stream
// of an iteration (the idea of xx16's packed DSPMV storage,
// src/programs/dev/xx16/xx16.f90:393-459).  The entries are stored by cyclic
// diagonals (packed_off): D[s][i] = K(i, (i+s) mod 60).
//
// Kernel structure (one persistent CTA of 12-14 warps per SM):
//   * every warp owns a ring of NSTAGE shared-memory stages with one
//     mbarrier each; lane 0 issues cp.async.bulk of the next elements'
//     packed blocks into the ring (complete_tx on the stage's mbarrier);
//   * the warp gathers p for the next element in registers, so the global
//     gather overlaps the current element's arithmetic;
//   * lane l < 30 owns rows l and l+30.  Forward distance d and backward
//     distance 30-d of both rows read D[d][l], D[d][l+30], D[30-d][l+d] and
//     D[30-d][(l+d+30) mod 60] with the p values l+d and l+d+30, so every
//     shared-memory address is the lane plus a compile-time constant and
//     each p load feeds two FMAs;
//   * the product is P K_e P p_e, P removing the element's mean translation
//     (an identity in exact arithmetic, since K_e annihilates rigid
//     translations).  It keeps the rounding of FP32 away from the smooth,
//     low-energy part of p, which otherwise slows the mixed solver's
//     convergence more the finer the mesh.  Rows l and l+30 share a
//     direction, so each mean is one reduction over the lanes of a class
//     mod 3.
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
constexpr int kPSlot = 120;                   // floats of p per warp (p_e twice)
constexpr unsigned kFull = 0xffffffffu;

}  // namespace

// Packs the FP64 storkm into the cyclic-diagonal FP32 layout of
// packed_off (one warp per element).
__global__ void k_pack_sym32(int nels, const double *__restrict__ km, float *__restrict__ kp)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int e = warp; e < nels; e += nwarps) {
        const double *ke = km + (size_t)e * 3600;
        float *out = kp + (size_t)e * kPacked;
        for (int pos = lane; pos < kPacked; pos += 32) {
            const int sd = pos < 1800 ? pos / 60 : 30, i = pos < 1800 ? pos % 60 : pos - 1800;
            out[pos] = pos < 1830 ? (float)ke[60 * ((i + sd) % 60) + i] : 0.0f;   // K(i, i+s)
        }
    }
}

// u_e = P K_e P p_e for every element, K_e from the packed FP32 diagonals.
// kWarps warps per CTA, kStages shared-memory stages per warp (tuned at
// run time among the instantiations below).  kMapped kernels (serving
// batches) read element numbers through emap; the solver's carry no
// remapping.
template <int kWarps, int kStages, bool kMapped>
__global__ void __launch_bounds__(kWarps * 32, 1)
k_elem_sym32(int nels, const float *__restrict__ kp, const int *__restrict__ conn,
             const double *__restrict__ p, float *__restrict__ ut, const PcgState *__restrict__ st,
             int *__restrict__ err, const int *__restrict__ emap)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    float *stage = reinterpret_cast<float *>(smem) + (size_t)w * kStages * kPacked;
    // p_e twice over (120 floats), so that (i + s) mod 60 needs no wrap
    float *pp = reinterpret_cast<float *>(smem + (size_t)kWarps * kStages * kPackedBytes) + w * kPSlot;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + (size_t)kWarps * kStages * kPackedBytes +
                                                 kWarps * kPSlot * 4) + w * kStages;
    static_assert((kWarps * kStages * kPackedBytes + kWarps * kPSlot * 4) % 8 == 0, "mbarrier alignment");

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
    auto elem = [&](int k) {
        const int g = first + k * kWarps;
        if constexpr (kMapped) return __ldg(emap + g);
        else return g;
    };

    if (lane == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    // storkm and the results pass through L2 once: evict them first, so that
    // p, which every element around a node gathers, stays in L2
    const uint64_t pol = l2_evict_first_policy();
    if (lane == 0) {
        for (int s = 0; s < kStages && s < nmine; ++s) {
            mbar_expect_tx(&bar[s], kPackedBytes);
            bulk_g2s_hint(stage + s * kPacked, kp + (size_t)elem(s) * kPacked, kPackedBytes, &bar[s], pol);
        }
    }

    // Lane l < 30 owns dofs and rows l and l+30 (node l/3 and node l/3+10,
    // both in direction l%3).  Gather pipeline: p of element k in registers
    // (FP64), connectivity of element k+1.
    const bool active = lane < 30;
    auto gather = [&](int nd, double &a, double &b) {
        const int n0 = __shfl_sync(kFull, nd, lane / 3);
        const int n1 = __shfl_sync(kFull, nd, active ? lane / 3 + 10 : 0);
        a = active ? p[(size_t)3 * n0 + lane % 3] : 0.0;
        b = active ? p[(size_t)3 * n1 + lane % 3] : 0.0;
    };
    int conn_next = 0;
    double pa = 0.0, pb = 0.0;
    {
        const int nd0 = lane < 20 ? conn[(size_t)elem(0) * 20 + lane] : 0;
        gather(nd0, pa, pb);
        if (nmine > 1 && lane < 20) conn_next = conn[(size_t)elem(1) * 20 + lane];
    }

    bool failed = false;
    int k = 0;
    for (; k < nmine; ++k) {
        const int s = k % kStages;
        const uint32_t parity = (uint32_t)((k / kStages) & 1);
        // prefetch: p of element k+1, connectivity of element k+2
        double na = 0.0, nb = 0.0;
        if (k + 1 < nmine) gather(conn_next, na, nb);
        int conn_next2 = 0;
        if (k + 2 < nmine && lane < 20) conn_next2 = conn[(size_t)elem(k + 2) * 20 + lane];

        // p of element k, less its mean translation, into the warp's slot.
        // K_e t = 0 for a rigid translation t, so the subtraction changes
        // nothing in exact arithmetic; in FP32 it keeps the translation of
        // a smooth p out of the rounding of p, of storkm's entries and of
        // the sums (errors that grow with the square of the mesh size on
        // the lowest modes).  The mean is formed from the FP32 high parts --
        // any translation serves -- and (hi - t) + lo recovers p - t to FP32
        // accuracy relative to p - t.
        {
            float ha, la, hb, lb;
            split_f64(pa, ha, la);
            split_f64(pb, hb, lb);
            const float t = 0.05f * sum_mod3(ha + hb, lane);
            if (active) {
                const float qa = (ha - t) + la, qb = (hb - t) + lb;
                pp[lane] = qa;
                pp[lane + 60] = qa;
                pp[lane + 30] = qb;
                pp[lane + 90] = qb;
            }
        }
        const bool ok = __all_sync(kFull, mbar_wait(&bar[s], parity));
        if (!ok) {
            failed = true;
            break;
        }
        __syncwarp();
        // Row l and row l+30 as four running sums over the diagonals: step
        // d pairs forward distance d (K(l, l+d), K(l+30, l+30+d)) with
        // backward distance 30-d (K(l+30, l+d), K(l, l+30+d)), which use
        // the same two p values.  Every address is the lane plus a constant.
        const float *D = stage + s * kPacked;
        float acc_a = 0.f, acc_b = 0.f;
        if (active) {
            const float *Dl = D + lane, *Dw = D + lane + 60;   // Dw: entries (l - t) mod 60 for t > l
            const float *pl = pp + lane;
            float f0 = Dl[0] * pl[0], f1 = Dl[30] * pl[30], g0 = 0.f, g1 = 0.f;
#pragma unroll
            for (int d = 1; d < 30; ++d) {
                const int t = 30 - d;
                const float p0 = pl[d], p1 = pl[30 + d];
                f0 = fmaf(Dl[60 * d], p0, f0);                              // K(l, l+d)
                f1 = fmaf(Dl[60 * d + 30], p1, f1);                         // K(l+30, l+30+d)
                g1 = fmaf(Dl[60 * t + d], p0, g1);                          // K(l+30, l+d) = D[t][l+d]
                g0 = fmaf((lane < t ? Dw : Dl)[59 * t], p1, g0);            // K(l, l-t) = D[t][(l-t) mod 60]
            }
            const float d30 = Dl[1800];                                     // K(l, l+30)
            f0 = fmaf(d30, pl[30], f0);
            f1 = fmaf(d30, pl[0], f1);
            acc_a = f0 + g0;
            acc_b = f1 + g1;
        }
        // the same projection on the result (t'K_e = 0 as well), so that
        // the product stays symmetric: u_e = P K_e P p_e
        {
            const float t = 0.05f * sum_mod3(acc_a + acc_b, lane);
            acc_a -= t;
            acc_b -= t;
        }
        if (active) {
            float *o = ut + (size_t)elem(k) * 80;   // node-padded: row i at (i/3)*4 + i%3
            st_global_hint(o + (lane / 3) * 4 + lane % 3, acc_a, pol);
            st_global_hint(o + (lane / 3 + 10) * 4 + lane % 3, acc_b, pol);
            // and the padding words, so that every 32-byte sector of the
            // results is written whole (a partly written one costs L2 a
            // read from DRAM once the results outgrow it)
            if (lane < 20) st_global_hint(o + lane * 4 + 3, 0.0f, pol);
        }
        __syncwarp();   // every lane is done with stage s and the p slot
        if (lane == 0 && k + kStages < nmine) {
            fence_proxy_async();
            mbar_expect_tx(&bar[s], kPackedBytes);
            bulk_g2s_hint(stage + s * kPacked, kp + (size_t)elem(k + kStages) * kPacked, kPackedBytes, &bar[s],
                          pol);
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
    return (size_t)W * S * kPackedBytes + W * kPSlot * 4 + W * S * 8;
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
        e = cudaFuncSetAttribute(k_elem_sym32<W, S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) {
            set_error("k_elem_sym32: cannot reserve %zu bytes of shared memory: %s", smem, cudaGetErrorString(e));
            return 1;
        }
        c.sym_attr |= bit;
    }
    const int grid = c.nels < c.nsm * W ? (c.nels + W - 1) / W : c.nsm;
    k_elem_sym32<W, S, false><<<grid, W * 32, smem, c.stream>>>(c.nels, c.km32p, c.conn, p, (float *)c.utemp, st,
                                                                c.kerr, nullptr);
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
    const cudaError_t e = cudaFuncSetAttribute(k_elem_sym32<14, 2, true>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
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
    k_elem_sym32<W, 2, true><<<grid, W * 32, sym_smem_bytes<W, 2>(), stream>>>(n, kp, conn, p, ut, nullptr, err,
                                                                                emap);
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
