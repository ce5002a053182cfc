// pf_elem_h16.cu -- element products from packed-symmetric FP16 storkm
// (PF_MODE_MIXED16 and pf_ebe_matvec prec 16).
//
// The inner PCG's products stream storkm from HBM once per iteration, so
// halving its bytes halves the dominant traffic of an iteration.  Each
// element's storkm is scaled by s_e = max |K_e| and rounded to FP16 (relative
// rounding 2^-11).  The FP64 defect correction of the mixed solver still
// brings the solve to the FP64 answer; the coarser operator costs inner
// iterations (100^3 cube: about 1.3x those of FP32 storage).  The product is
// translation-projected (P K_e P p_e), as the FP32 kernel's is: without the
// projection the FP16 rounding of K_e t would dominate the lowest modes.
//
// Storage per element (916 words = 3,664 bytes, a multiple of 16): the
// cyclic diagonals D[s][i] = K(i, (i+s) mod 60) / s_e of packed_off, s =
// 0..29, as 30 half2 words per diagonal, word 30s + m = (D[s][m], D[s][m+30]);
// then diagonal 30's entries K(i, i+30) / s_e, i = 0..29, as halves 1800..1829
// (words 900..914); then s_e as an FP32 (word 915).  Lane l owns rows l and
// l+30, and every step of the walk over the diagonals reads one word per
// lane: forward distance d needs (D[d][l], D[d][l+30]) = word 30d + l, and
// backward distance t = 30 - d needs D[t][l+d] and D[t][(l+d+30) mod 60],
// the two halves of word 30t + (l+d) mod 30 (swapped when l+d >= 30).
#include "pf_internal.h"
#include "pf_tc.cuh"

#include <cstdint>
#include <cuda_fp16.h>

namespace pf {

using namespace tc;

namespace {
constexpr int kH16Words = 916;
constexpr int kH16Bytes = kH16Words * 4;   // 3664
constexpr int kPSlot = 120;                // floats of p per warp: 60 pairs (p[i], p[i+30 mod 60])
constexpr unsigned kFull = 0xffffffffu;
}  // namespace

// Packs the FP64 storkm into the FP16 layout above (one warp per element).
__global__ void k_pack_sym16(int nels, const double *__restrict__ km, uint32_t *__restrict__ kh)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int e = warp; e < nels; e += nwarps) {
        const double *ke = km + (size_t)e * 3600;
        uint32_t *out = kh + (size_t)e * kH16Words;
        double mx = 0.0;
        for (int q = lane; q < 3600; q += 32) mx = fmax(mx, fabs(ke[q]));
        for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(kFull, mx, o));
        const double inv = mx > 0.0 ? 1.0 / mx : 0.0;
        for (int w = lane; w < 900; w += 32) {   // diagonals 0..29: (D[s][m], D[s][m+30])
            const int sd = w / 30, m = w % 30;
            const float lo = (float)(ke[60 * ((m + sd) % 60) + m] * inv);            // K(m, m+s)
            const float hi = (float)(ke[60 * ((m + 30 + sd) % 60) + m + 30] * inv);  // K(m+30, m+30+s)
            const __half2 h = __floats2half2_rn(lo, hi);
            out[w] = *reinterpret_cast<const uint32_t *>(&h);
        }
        if (lane < 15) {                          // diagonal 30: K(i, i+30), i = 2 lane, 2 lane + 1
            const int i = 2 * lane;
            const __half2 h = __floats2half2_rn((float)(ke[60 * (i + 30) + i] * inv),
                                                (float)(ke[60 * (i + 31) + i + 1] * inv));
            out[900 + lane] = *reinterpret_cast<const uint32_t *>(&h);
        }
        if (lane == 0) out[915] = __float_as_uint((float)mx);
    }
}

// u_e = P K_e P p_e for every element, K_e from the FP16 diagonals.
// kWarps warps per CTA, kStages shared-memory stages per warp, p gathered
// kAhead (1 or 2) elements ahead of the one being multiplied.  kMapped
// kernels (serving batches) read element numbers through emap; the solver's
// kernels carry no remapping (a runtime test cost the 20-warp configuration
// 14 % of its time).
template <int kWarps, int kStages, int kAhead, bool kMapped>
__global__ void __launch_bounds__(kWarps * 32, 1)
k_elem_sym16(int nels, const uint32_t *__restrict__ kh, const int *__restrict__ conn,
             const double *__restrict__ p, float *__restrict__ ut, const PcgState *__restrict__ st,
             int *__restrict__ err, const int *__restrict__ emap)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    uint32_t *stage = reinterpret_cast<uint32_t *>(smem) + (size_t)w * kStages * kH16Words;
    float2 *pp = reinterpret_cast<float2 *>(smem + (size_t)kWarps * kStages * kH16Bytes + (size_t)w * kPSlot * 4);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + (size_t)kWarps * kStages * kH16Bytes +
                                                 kWarps * kPSlot * 4) + w * kStages;
    static_assert((kWarps * kStages * kH16Bytes + kWarps * kPSlot * 4) % 8 == 0, "mbarrier alignment");

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
    const int nmine = (e1 - first + kWarps - 1) / kWarps;
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
            mbar_expect_tx(&bar[s], kH16Bytes);
            bulk_g2s_hint(stage + s * kH16Words, kh + (size_t)elem(s) * kH16Words, kH16Bytes, &bar[s], pol);
        }
    }

    const bool active = lane < 30;
    auto gather = [&](int nd, double &a, double &b) {
        const int n0 = __shfl_sync(kFull, nd, lane / 3);
        const int n1 = __shfl_sync(kFull, nd, active ? lane / 3 + 10 : 0);
        a = active ? p[(size_t)3 * n0 + lane % 3] : 0.0;
        b = active ? p[(size_t)3 * n1 + lane % 3] : 0.0;
    };
    // p of elements k (pa, pb) and, for kAhead 2, k+1 (qa, qb); conn_next
    // holds the connectivity of element k + kAhead
    int conn_next = 0;
    double pa = 0.0, pb = 0.0, qa = 0.0, qb = 0.0;
    {
        const int nd0 = lane < 20 ? conn[(size_t)elem(0) * 20 + lane] : 0;
        gather(nd0, pa, pb);
        if (kAhead == 2 && nmine > 1) {
            const int nd1 = lane < 20 ? conn[(size_t)elem(1) * 20 + lane] : 0;
            gather(nd1, qa, qb);
        }
        if (nmine > kAhead && lane < 20) conn_next = conn[(size_t)elem(kAhead) * 20 + lane];
    }

    bool failed = false;
    int k = 0;
    for (; k < nmine; ++k) {
        const int s = k % kStages;
        const uint32_t parity = (uint32_t)((k / kStages) & 1);
        double na = 0.0, nb = 0.0;   // p of element k + kAhead
        if (k + kAhead < nmine) gather(conn_next, na, nb);
        int conn_next2 = 0;
        if (k + kAhead + 1 < nmine && lane < 20) conn_next2 = conn[(size_t)elem(k + kAhead + 1) * 20 + lane];

        // p of element k less its mean translation (as the FP32 kernel)
        {
            float ha, la, hb, lb;
            split_f64(pa, ha, la);
            split_f64(pb, hb, lb);
            const float t = 0.05f * sum_mod3(ha + hb, lane);
            if (active) {   // pair i = (p[i], p[i+30 mod 60]): one 8-byte load per step of the walk
                const float qa = (ha - t) + la, qb = (hb - t) + lb;
                pp[lane] = make_float2(qa, qb);
                pp[lane + 30] = make_float2(qb, qa);
            }
        }
        const bool ok = __all_sync(kFull, mbar_wait(&bar[s], parity));
        if (!ok) {
            failed = true;
            break;
        }
        __syncwarp();
        const uint32_t *Wd = stage + s * kH16Words;
        float acc_a = 0.f, acc_b = 0.f;
        if (active) {
            const float2 *pl = pp + lane;
            const float2 p00 = pl[0];   // (p[l], p[l+30])
            const float2 w0 = __half22float2(*reinterpret_cast<const __half2 *>(Wd + lane));
            float f0 = w0.x * p00.x, f1 = w0.y * p00.y, g0 = 0.f, g1 = 0.f;
#pragma unroll
            for (int d = 1; d < 30; ++d) {
                const int t = 30 - d;
                const float2 pd = pl[d];   // (p[l+d], p[l+d+30 mod 60])
                const float p0 = pd.x, p1 = pd.y;
                const float2 wf = __half22float2(*reinterpret_cast<const __half2 *>(Wd + 30 * d + lane));
                f0 = fmaf(wf.x, p0, f0);                                      // K(l, l+d)
                f1 = fmaf(wf.y, p1, f1);                                      // K(l+30, l+30+d)
                const bool wrap = lane >= t;                                  // l + d >= 30
                const float2 wb = __half22float2(
                    *reinterpret_cast<const __half2 *>(Wd + 30 * t + (wrap ? lane - t : lane + d)));
                g1 = fmaf(wrap ? wb.y : wb.x, p0, g1);                        // K(l+30, l+d)
                g0 = fmaf(wrap ? wb.x : wb.y, p1, g0);                        // K(l, l+d+30)
            }
            const float d30 = __half2float(reinterpret_cast<const __half *>(Wd + 900)[lane]);   // K(l, l+30)
            f0 = fmaf(d30, p00.y, f0);
            f1 = fmaf(d30, p00.x, f1);
            const float sc = __uint_as_float(Wd[915]);
            acc_a = (f0 + g0) * sc;
            acc_b = (f1 + g1) * sc;
        }
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
            mbar_expect_tx(&bar[s], kH16Bytes);
            bulk_g2s_hint(stage + s * kH16Words, kh + (size_t)elem(k + kStages) * kH16Words, kH16Bytes, &bar[s],
                          pol);
        }
        if (kAhead == 2) {
            pa = qa;
            pb = qb;
            qa = na;
            qb = nb;
        } else {
            pa = na;
            pb = nb;
        }
        conn_next = conn_next2;
    }
    if (failed) {
        if (lane == 0) atomicExch(err, 2);
        for (int kk = k; kk < nmine && kk < k + kStages; ++kk)
            mbar_wait(&bar[kk % kStages], (uint32_t)((kk / kStages) & 1));
    }
}

template <int W, int S>
constexpr size_t h16_smem_bytes()
{
    return (size_t)W * S * kH16Bytes + W * kPSlot * 4 + W * S * 8;
}

template <int W, int S, int A>
static int launch_h16_cfg(Ctx &c, const double *p, const PcgState *st, int bit)
{
    constexpr size_t smem = h16_smem_bytes<W, S>();
    static_assert(smem <= 227 * 1024, "shared memory per CTA");
    cudaError_t e;
    if (!(c.h16_attr & (1u << bit))) {   // once per context and configuration, before any stream capture
        e = cudaFuncSetAttribute(k_elem_sym16<W, S, A, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) {
            set_error("k_elem_sym16: cannot reserve %zu bytes of shared memory: %s", smem, cudaGetErrorString(e));
            return 1;
        }
        c.h16_attr |= 1u << bit;
    }
    const int grid = c.nels < c.nsm * W ? (c.nels + W - 1) / W : c.nsm;
    k_elem_sym16<W, S, A, false><<<grid, W * 32, smem, c.stream>>>(c.nels, c.km16p, c.conn, p, (float *)c.utemp,
                                                                   st, c.kerr, nullptr);
    c.launches++;
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_elem_sym16: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

// the tuned configurations: (warps per CTA, stages per warp); half the
// bytes per stage of the FP32 kernel, so more warps fit and hide the latency
// of the p gather.  The 20- and 24-warp configurations gather p two
// elements ahead (90 and 78 registers), the 28-warp one, at 70 registers,
// one element ahead.
static const int kH16Cfg[][2] = {{20, 2}, {24, 2}, {28, 2}};
constexpr int kNumH16Cfg = 3;

static int launch_h16_index(Ctx &c, int idx, const double *p, const PcgState *st)
{
    switch (idx) {
    case 1: return launch_h16_cfg<24, 2, 2>(c, p, st, 1);
    case 2: return launch_h16_cfg<28, 2, 1>(c, p, st, 2);
    default: return launch_h16_cfg<20, 2, 2>(c, p, st, 0);
    }
}

// The FP16 packed storkm of the context, packed from the FP64 storkm on the
// first use after storkm was formed or set, and its configuration autotuned
// (as the FP32 kernel's: one warm-up and three timed launches each).
int ensure_km16(Ctx &c)
{
    if (c.km16_ok) return 0;
    if (!c.km64) {
        set_error("FP16 products: the context holds no per-element storkm");
        return 1;
    }
    if (!c.km16p) {
        if (cudaMalloc((void **)&c.km16p, (size_t)c.nels * kH16Bytes) != cudaSuccess) {
            cudaGetLastError();
            set_error("FP16 products: cannot allocate %zu bytes of packed storkm", (size_t)c.nels * kH16Bytes);
            return 1;
        }
    }
    k_pack_sym16<<<c.nsm * 8, 256, 0, c.stream>>>(c.nels, c.km64, c.km16p);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_pack_sym16: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        set_error("FP16 autotune: cannot create events");
        return 1;
    }
    float best = 1e30f;
    int best_i = 0;
    for (int i = 0; i < kNumH16Cfg; ++i) {
        if (launch_h16_index(c, i, c.x, nullptr)) return 1;
        cudaEventRecord(a, c.stream);
        for (int r = 0; r < 3; ++r)
            if (launch_h16_index(c, i, c.x, nullptr)) return 1;
        cudaEventRecord(b, c.stream);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        c.tune16_ms[i] = ms / 3.0f;
        if (ms < best) {
            best = ms;
            best_i = i;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    c.h16_cfg = best_i;
    c.km16_ok = true;
    return 0;
}

int launch_elem_sym16(Ctx &c, const double *p, const PcgState *st)
{
    return launch_h16_index(c, c.h16_cfg, p, st);
}

// The serving engine's entry points: the (20, 2, 2) configuration over n
// active elements mapped to arena elements by emap.  sym16_prepare sets the
// shared-memory attribute; call it once per device before any stream capture.
int sym16_prepare()
{
    constexpr size_t smem = h16_smem_bytes<20, 2>();
    const cudaError_t e = cudaFuncSetAttribute(k_elem_sym16<20, 2, 2, true>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
        set_error("k_elem_sym16: cannot reserve %zu bytes of shared memory: %s", smem, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int launch_elem_sym16_mapped(cudaStream_t stream, int nsm, int n, const uint32_t *kh, const int *conn,
                             const double *p, float *ut, int *err, const int *emap)
{
    if (n <= 0) return 0;
    constexpr int W = 20;
    const int grid = n < nsm * W ? (n + W - 1) / W : nsm;
    k_elem_sym16<W, 2, 2, true><<<grid, W * 32, h16_smem_bytes<W, 2>(), stream>>>(n, kh, conn, p, ut, nullptr, err,
                                                                                   emap);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_elem_sym16: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int launch_pack_sym16_raw(cudaStream_t stream, int nsm, int nels, const double *km, uint32_t *kh)
{
    k_pack_sym16<<<nsm * 8, 256, 0, stream>>>(nels, km, kh);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_pack_sym16: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

int h16_config(int idx, int *warps, int *stages)
{
    if (idx < 0 || idx >= kNumH16Cfg) return 1;
    *warps = kH16Cfg[idx][0];
    *stages = kH16Cfg[idx][1];
    return 0;
}

}  // namespace pf
