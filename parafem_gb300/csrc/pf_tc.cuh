// pf_tc.cuh -- inline-PTX helpers for the Blackwell asynchronous units:
// mbarriers, bulk copies (cp.async.bulk, the TMA engine without a tensor
// map), tcgen05 tensor-core MMAs with TMEM accumulators, and the BF16
// three-term split used to reach FP32 accuracy on BF16 tensor cores.
//
// Every wait here is bounded: mbar_wait returns false after kSpinLimit polls
// (each poll suspends the thread for at most kSuspendNs nanoseconds, so a
// wait gives up after about four seconds) and the caller records an error
// and drains what it has in flight.
#pragma once
#include <cstdint>

namespace pf {
namespace tc {

constexpr long long kSpinLimit = 1LL << 22;   // try_wait polls before giving up
constexpr uint32_t kSuspendNs = 1000;          // longest suspension of one poll

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---------------------------------------------------------------------------
// mbarriers
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// arrive once and expect `bytes` of transaction (bulk-copy) completions
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kSuspendNs)
        : "memory");
    return ok != 0;
}

// Non-blocking test of the phase with the given parity: independent tests
// of several barriers overlap their shared-memory round trips.
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity: false when `limit`
// polls ran out.
__device__ __forceinline__ bool mbar_wait_n(uint64_t *bar, uint32_t parity, long long limit)
{
    for (long long i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) { return mbar_wait_n(bar, parity, kSpinLimit); }

// ---------------------------------------------------------------------------
// bulk copies global -> shared (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// L2 policy for data a kernel touches once (streamed storkm, element
// results): its lines are the first evicted, so that a vector gathered many
// times (p) keeps its lines in L2 while gigabytes stream past.
__device__ __forceinline__ uint64_t l2_evict_first_policy()
{
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// bulk_g2s with an L2 cache policy (l2_evict_first_policy)
__device__ __forceinline__ void bulk_g2s_hint(void *dst, const void *src, uint32_t bytes, uint64_t *bar,
                                              uint64_t pol)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}

// 4-byte global store with an L2 cache policy
__device__ __forceinline__ void st_global_hint(float *dst, float v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(dst), "f"(v), "l"(pol) : "memory");
}

// 16-byte copy global -> shared that bypasses L1 (cp.async, both addresses
// 16-byte aligned); completion is tracked per thread, see cp_async_arrive
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

// The mbarrier receives one arrival when every cp.async this thread issued
// so far has completed.  The barrier's pending count is raised by one first,
// so the arrival leaves the count the phase expects unchanged: issue it
// before the phase's last ordinary arrival.
__device__ __forceinline__ void cp_async_arrive(uint64_t *bar)
{
    asm volatile("cp.async.mbarrier.arrive.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// TMA gather: four rows (y0..y3) of a 2-D tensor, each the tensor map's box
// (one row high) starting at column x, to consecutive places in shared
// memory (dst 128-byte aligned; x * element size a multiple of 16 bytes);
// completion counted in bytes on the mbarrier.  tmap is the generic address
// of a CUtensorMap kernel parameter.
__device__ __forceinline__ void tma_gather4(void *dst, const void *tmap, int x, int y0, int y1, int y2, int y3,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y0), "r"(y1), "r"(y2), "r"(y3), "r"(smem_u32(bar))
        : "memory");
}

// orders this thread's generic-proxy shared-memory accesses with the async proxy
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---------------------------------------------------------------------------
// tcgen05
// Shared-memory matrix descriptor, K-major, no swizzle: core matrices of
// 8 rows x 16 bytes stored contiguously; LBO = byte distance between core
// matrices adjacent in K, SBO = between core matrices adjacent in M/N.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version 1 (sm_100 family); base offset 0; no swizzle
    return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// Instruction descriptor, kind::f16: D = F32, A = B = F16 (format code 0),
// both K-major.  n may be a run-time value (a multiple of 8).
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t m, uint32_t n)
{
    return (1u << 4) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// the mbarrier completes when every MMA this thread issued so far has finished
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// whole-warp TMEM allocation of `ncols` columns (a power of two >= 32); the
// base address is written to *slot
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t base, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Four 8x8 16-bit matrices between shared memory and registers: ldmatrix
// with .trans hands each thread its fragment of the transposed matrices,
// stmatrix writes fragments back as rows.  Thread i gives the address of row
// i % 8 of matrix i / 8 (16 bytes, 16-byte aligned).
__device__ __forceinline__ void ldsm_x4_trans(uint32_t addr, uint32_t (&r)[4])
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr)
                 : "memory");
}

__device__ __forceinline__ void stsm_x4(uint32_t addr, const uint32_t (&r)[4])
{
    asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(r[0]), "r"(r[1]),
                 "r"(r[2]), "r"(r[3])
                 : "memory");
}

// Two floats rounded to nearest-even FP16 in one instruction: lo in bits
// 0..15, hi in bits 16..31.
__device__ __forceinline__ uint32_t cvt_f16x2(float lo, float hi)
{
    uint32_t r;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes (lane = row)
__device__ __forceinline__ void tmem_ld_32x32b_x16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive columns of this warp's 32 TMEM lanes (one lane per thread),
// the load and its wait in one statement
__device__ __forceinline__ void tmem_ld_32x32b_x32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// FP64 -> FP32 high + low parts without the FP64 pipe
// v = hi + lo with hi = v truncated to FP32 and lo the FP32 remainder
// (rounded to 23 bits), by integer operations on the bits of v.  GB300's FP64
// rate is about 1/60 of its FP32 rate; this takes FP64 vectors into FP32
// kernels with no FP64 arithmetic and no FP64 conversion.  |hi + lo - v| <= 2^-46 |v| for 2^-103 <= |v| <
// 2^128; below that lo is 0 (hi alone is accurate to 2^-23), |v| >= 2^128
// gives hi = +-inf and a NaN gives a NaN.
__device__ __forceinline__ void split_f64(double v, float &hi, float &lo)
{
    const uint32_t bh = (uint32_t)__double2hiint(v), bl = (uint32_t)__double2loint(v);
    const uint32_t sign = bh & 0x80000000u;
    const int e = (int)((bh >> 20) & 0x7ffu);          // biased FP64 exponent
    const int fe = e - 1023 + 127;                      // biased FP32 exponent
    const uint32_t mant = ((bh & 0xfffffu) << 3) | (bl >> 29);
    if (fe >= 1 && fe <= 254)
        hi = __uint_as_float(sign | ((uint32_t)fe << 23) | mant);
    else if (fe > 254)
        hi = __uint_as_float(sign | 0x7f800000u | ((e == 0x7ff && ((bh & 0xfffffu) | bl)) ? 0x400000u : 0u));
    else
        hi = __uint_as_float(sign);
    // the low 29 mantissa bits, top 23 of them: (rem >> 6) * 2^(e - 1069)
    const float m = __uint_as_float(0x3f800000u | ((bl & 0x1fffffffu) >> 6)) - 1.0f;   // (rem >> 6) * 2^-23
    const int se = e - 1046 + 127;                                                     // 2^(e - 1046)
    lo = (fe >= 1 && se >= 1 && se <= 254)
             ? __uint_as_float(__float_as_uint(m * __uint_as_float((uint32_t)se << 23)) | sign)
             : 0.0f;
}

// Sums v over each class of lanes with equal index mod 3 (lanes 0..29 hold
// the values, lanes 30 and 31 hold 0) and returns to every lane the sum of
// its class, the same bits on every lane of the class.
__device__ __forceinline__ float sum_mod3(float v, int lane)
{
#pragma unroll
    for (int off = 3; off < 32; off <<= 1) {   // 3, 6, 12, 24
        const float w = __shfl_down_sync(0xffffffffu, v, off);
        v += (lane + off < 32) ? w : 0.0f;
    }
    return __shfl_sync(0xffffffffu, v, lane % 3);
}

// ---------------------------------------------------------------------------
// BF16 three-term split
// Two floats rounded to nearest-even BF16 in one instruction: lo in bits
// 0..15, hi in bits 16..31.
__device__ __forceinline__ uint32_t cvt_bf16x2(float lo, float hi)
{
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// Splits 8 consecutive K-values into three BF16 terms (x = h1 + h2 + h3;
// each remainder is exact in FP32) and writes the three 16-byte chunks, one
// per term tile (term t at dst + t * term_bytes).  Each term is the
// nearest-even BF16 of the remainder left by the terms before it.
__device__ __forceinline__ void split3_store8(const float (&x)[8], unsigned char *dst, uint32_t term_bytes)
{
    uint32_t w1[4], w2[4], w3[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const float a = x[2 * r], b = x[2 * r + 1];
        w1[r] = cvt_bf16x2(a, b);
        const float ra = a - __uint_as_float(w1[r] << 16), rb = b - __uint_as_float(w1[r] & 0xFFFF0000u);
        w2[r] = cvt_bf16x2(ra, rb);
        const float sa = ra - __uint_as_float(w2[r] << 16), sb = rb - __uint_as_float(w2[r] & 0xFFFF0000u);
        w3[r] = cvt_bf16x2(sa, sb);
    }
    *reinterpret_cast<uint4 *>(dst) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
    *reinterpret_cast<uint4 *>(dst + term_bytes) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
    *reinterpret_cast<uint4 *>(dst + 2 * term_bytes) = make_uint4(w3[0], w3[1], w3[2], w3[3]);
}

// byte offset of (row, k) in a K-major no-swizzle tile with 64 K-columns:
// 8-row groups 1024 B apart (SBO), 8-column core matrices 128 B apart (LBO)
__device__ __forceinline__ uint32_t kmajor_off(int row, int k)
{
    return (uint32_t)((row >> 3) * 1024 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

}  // namespace tc
}  // namespace pf
