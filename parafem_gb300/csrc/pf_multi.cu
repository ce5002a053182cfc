// pf_multi.cu -- k load cases of one mesh solved together (block PCG).
//
// k independent Jacobi-PCG solves (p121.f90:86-104) share every element
// matrix read: one iteration computes U = K P for a 60 x k block per element.
// Vectors are interleaved per slot, v[slot*k + j], so the gather of an
// element's block and the node scatter touch k consecutive values.
//
// Element products:
//   k_mr_elem_tc   tensor cores (tcgen05.mma, kind::f16, BF16 operands, FP32
//                  accumulation in TMEM), operands from the packed-symmetric
//                  FP32 storkm by bulk copy.  K_e and P_e are each split into
//                  three BF16 terms (x = h1 + h2 + h3, about 24 significant
//                  bits) and the six products of order <= 2^-16 are summed:
//                  the block product reaches FP32 accuracy.  A two-term split
//                  (about 16 bits) leaves too large a perturbation of K for
//                  the inner PCG to converge on these meshes.
//   k_mr_elem_cc   the same product on CUDA cores in FP32 (check and fallback
//                  kernel for the tensor-core one, selectable by prec).
//   k_mr_elem_64   FP64 (DFMA) block product for the true residual f - K x.
// The inner PCG runs on the FP32-class product with FP64 vectors, dots and
// alpha/beta; the recursive residuals are replaced by the FP64 true residual
// whenever an active load case has dropped 10x (as PF_MODE_MIXED does).
#include "pf_device.cuh"
#include "pf_tc.cuh"
#include "pfgpu.h"

#include <cstring>
#include <vector>

namespace pf {

using namespace tc;

namespace {

constexpr int KR = 16;               // load cases per block (the kernels are written for 16)
constexpr unsigned kFullMask = 0xffffffffu;

// Tile geometry (BF16, K-major, no swizzle; 8-row x 16-byte core matrices,
// LBO = 128 B between core matrices adjacent in K, SBO = 1024 B between
// 8-row groups).  A term holds 96 rows: for direction d, rows 32d + i
// (i < 20) are K_e's rows 3i + d, row 32d + 20 is the sum of those rows, rows
// 32d + 21..31 stay zero.  The MMA reads M = 128 rows, so rows 96..127 of a
// term are the next 4 KB of shared memory: they only feed accumulator rows
// 96..127, which nobody reads.
constexpr int kRowsA = 96;
constexpr int kTermA = kRowsA * 64 * 2;      // 12288
constexpr int kBufA = 3 * kTermA + 4096;     // 3 terms + the 4 KB read as rows 96..127 of the last
constexpr int kTermB = 16 * 64 * 2;          // 2048: 16 load cases x 64 K
constexpr int kBufB = 3 * kTermB;
constexpr int kStK = 7328;                   // packed-symmetric FP32 K_e (1830 + 2 pad floats)
constexpr int kStP = 20 * 3 * KR * 8;        // P of the 20 nodes: 20 x 384 B
constexpr int kStC = 3 * 64 * 4;             // direction sums of K_e's rows (3 x 64 FP32)
constexpr int kStage = kStK + kStP + kStC;   // 15776 B, a multiple of 16
constexpr int kNst = 4;                      // operand stages (bulk copies in flight)
constexpr int kNTile = 3;                    // BF16 tile sets (A + B)
constexpr int kNAcc = 4;                     // TMEM accumulators (16 columns each)
constexpr int kBuildWarps = 16;              // warps 0-15 split K_e and P_e
constexpr int kGroups = 2;                   // builder groups: warps 8g..8g+7 build the elements t = g mod 2
constexpr int kGroupWarps = kBuildWarps / kGroups;
constexpr int kBWarps = 4;                   // warps 8g..8g+3 also split P_e (one B task per thread)
constexpr int kEpiWarp0 = 16;                // warps 16-18 read TMEM lanes 32d..32d+31 back (direction d)
constexpr int kNEpi = 3;
constexpr int kProdWarp = 19;                // warp 19 issues the bulk copies
constexpr int kMmaWarp = 20;                 // warp 20, lane 0 issues the MMAs
constexpr int kTcThreads = 21 * 32;
static_assert(kGroupWarps * 32 * 2 >= 63 * 8, "two A tasks (row, 8 K-values) per builder thread");
static_assert(kBWarps * 32 == KR * 8, "one B task (load case, 8 dofs) per thread of a group's first four warps");
constexpr int kOffB = kNTile * kBufA;
constexpr int kOffSt = kOffB + kNTile * kBufB;
constexpr int kOffAux = kOffSt + kNst * kStage;
constexpr int kOffSum = kOffAux + 256;       // [group][2][8][KR][3] partial direction sums of P_e
constexpr int kTcSmem = kOffSum + kGroups * 2 * 8 * KR * 3 * 4;
constexpr uint32_t kIdesc = idesc_bf16(128, 16);
static_assert(kOffSt % 16 == 0 && kStage % 16 == 0 && kOffAux % 8 == 0, "bulk-copy alignment");
static_assert(kTcSmem <= 227 * 1024, "shared memory per CTA");
static_assert(kEpiWarp0 % 4 == 0, "epilogue warp kEpiWarp0 + d must reach TMEM lanes 32d..32d+31");

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

}  // namespace

// Block element products on the tensor cores: ut[e][i][j] = sum_c K_e(i,c) P(slot(c), j).
//
// The product is P K_e P P_e, P removing each load case's mean translation
// over the element's 20 nodes (an identity in exact arithmetic, since K_e
// annihilates rigid translations; in FP32-class arithmetic it keeps the
// rounding away from the smooth part of P, as the single-case kernels do).
//
// One persistent CTA of 21 warps per SM walks the elements e = blockIdx.x +
// t * gridDim.x with warp-specialised roles linked by mbarriers:
//   warp 19      bulk copies (cp.async.bulk) of the packed symmetric storkm of
//                K_e (7,328 B), of the 16-case P blocks of the element's
//                20 nodes (384 B each, contiguous in the interleaved vector)
//                and of the direction sums of K_e's rows (768 B) into a ring
//                of kNst stages;
//   warps 0-15   split K_e (rows by direction, with the row sums) and P_e
//                less its mean translations into three BF16 terms each and
//                write them into a ring of kNTile tile sets.  Two groups of
//                eight warps take alternate elements; a thread has two
//                8-value row segments of K_e (shared-memory offsets computed
//                once), and a group's warps 0-3 also one 8-dof segment of
//                P_e each, exchanging partial sums through shared memory;
//   warp 20      one thread issues the six products of order <= 2^-16
//                (24 MMAs, M=128, N=16, K=16) into a ring of kNAcc TMEM
//                accumulators and commits them to mbarriers that free the
//                tile set and fill the accumulator;
//   warps 16-18  read the accumulators back (TMEM lanes 32d..32d+20,
//                direction d), subtract the mean of the direction's rows and
//                store the 60 x 16 results.
// Every wait is bounded.  A wait that runs out sets a shared failure flag
// that every role checks before its next wait, writes 3 to the device error
// word, and the CTA waits (bounded) for the copies and MMAs it has in flight
// before it frees its TMEM and returns.
__global__ void __launch_bounds__(kTcThreads, 1)
k_mr_elem_tc(int nels, const float *__restrict__ kp, const float *__restrict__ ksum, const int *__restrict__ conn,
             const double *__restrict__ P, float *__restrict__ ut, int *__restrict__ err,
             const int *__restrict__ skip)
{
    if (skip && *skip) return;   // a residual replacement is pending: nothing to compute
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *A = sm;
    unsigned char *B = sm + kOffB;
    unsigned char *stg = sm + kOffSt;
    uint64_t *st_full = reinterpret_cast<uint64_t *>(sm + kOffAux);
    uint64_t *st_empty = st_full + kNst;
    uint64_t *tl_full = st_empty + kNst;
    uint64_t *tl_empty = tl_full + kNTile;
    uint64_t *ac_full = tl_empty + kNTile;
    uint64_t *ac_empty = ac_full + kNAcc;
    uint64_t *sum_bar = ac_empty + kNAcc;   // [group]: its four B warps' partial sums of an element are written
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sum_bar + kGroups);
    float *psum = reinterpret_cast<float *>(sm + kOffSum);   // [group][k & 1][chunk][case][direction]
    volatile int *s_fail = reinterpret_cast<volatile int *>(tslot + 1);
    int *s_count = reinterpret_cast<int *>(tslot + 2);   // [0] copies issued, [1] MMA groups committed
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nmine = blockIdx.x < nels ? (nels - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto elem = [&](int t) { return (int)blockIdx.x + t * (int)gridDim.x; };

    for (int i = tid; i < kOffSt / 16; i += kTcThreads) reinterpret_cast<uint4 *>(sm)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 0) tmem_alloc(tslot, 64);
    if (tid == 0) {
        for (int i = 0; i < kNst; ++i) {
            mbar_init(&st_full[i], 1);
            mbar_init(&st_empty[i], kGroupWarps);
        }
        for (int i = 0; i < kNTile; ++i) {
            mbar_init(&tl_full[i], kGroupWarps);
            mbar_init(&tl_empty[i], 1);
        }
        for (int i = 0; i < kNAcc; ++i) {
            mbar_init(&ac_full[i], 1);
            mbar_init(&ac_empty[i], kNEpi);
        }
        for (int g = 0; g < kGroups; ++g) mbar_init(&sum_bar[g], kBWarps);
        mbar_fence_init();
        *s_fail = 0;
        s_count[0] = s_count[1] = 0;
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    // bounded wait that also gives up at once when another role has failed
    auto wait = [&](uint64_t *bar, uint32_t parity) {
        if (*s_fail) return false;
        if (mbar_wait(bar, parity)) return true;
        *s_fail = 1;
        return false;
    };

    if (warp == kProdWarp) {
        // the connectivity (lane a: node a of the element) is loaded kCD
        // elements ahead, so its latency is not paid once per element
        constexpr int kCD = 8;
        int ndr[kCD];
#pragma unroll
        for (int j = 0; j < kCD; ++j) ndr[j] = (lane < 20 && j < nmine) ? conn[(size_t)elem(j) * 20 + lane] : 0;
        int issued = 0;   // elements whose copies are in flight or done
        bool stop = false;
        for (int t0 = 0; t0 < nmine && !stop; t0 += kCD) {
#pragma unroll
            for (int j = 0; j < kCD; ++j) {
                const int t = t0 + j;
                if (t >= nmine) break;
                const int s = t % kNst;
                if (t >= kNst && !wait(&st_empty[s], (uint32_t)((t / kNst - 1) & 1))) {
                    stop = true;
                    break;
                }
                unsigned char *dst = stg + s * kStage;
                if (lane == 0) mbar_expect_tx(&st_full[s], kStage);
                __syncwarp();
                if (lane == 0) bulk_g2s(dst, kp + (size_t)elem(t) * 1832, kStK, &st_full[s]);
                if (lane < 20) bulk_g2s(dst + kStK + lane * 384, P + (size_t)3 * ndr[j] * KR, 384, &st_full[s]);
                if (lane == 20) bulk_g2s(dst + kStK + kStP, ksum + (size_t)elem(t) * 192, kStC, &st_full[s]);
                ndr[j] = (lane < 20 && t + kCD < nmine) ? conn[(size_t)elem(t + kCD) * 20 + lane] : 0;
                issued = t + 1;
            }
        }
        if (lane == 0) s_count[0] = issued;
    } else if (warp < kBuildWarps) {
        // Two groups of eight warps build alternate elements, so two
        // elements are in the build stage at once.  A thread of a group has
        // two A tasks (of 504): A row 32d + i, K-values 8q..8q+7.  i < 20:
        // K(3i + d, k) at packed_off; i = 20: the sum of direction d's rows,
        // after the P blocks in the stage; K-values past 59 read the zero
        // pad at 1830.
        const int grp = warp / kGroupWarps, gw = warp % kGroupWarps, gtid = tid % (kGroupWarps * 32);
        int off[2][8];
        uint32_t a_off[2];
        bool a_task[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int task = gtid + h * kGroupWarps * 32;
            a_task[h] = task < 63 * 8;
            const int r63 = task % 63, q = task / 63;
            const int d = r63 / 21, i = r63 % 21;
#pragma unroll
            for (int g = 0; g < 8; ++g) {
                const int k = 8 * q + g;
                off[h][g] = (!a_task[h] || k >= 60) ? 1830
                            : i < 20                ? packed_off(3 * i + d, k)
                                                    : (kStK + kStP) / 4 + 64 * d + k;
            }
            a_off[h] = a_task[h] ? kmajor_off(32 * d + i, 8 * q) : 0u;
        }
        // B task (the group's warps 0-3): load case j, dofs 8qb..8qb+7 (dof c
        // has direction (rb + c - 8qb) % 3)
        const int j = gtid & (KR - 1), qb = gtid >> 4;
        const int rb = (2 * qb) % 3;
        const bool b_task = gw < kBWarps;
        uint64_t *my_sum = &sum_bar[grp];
        for (int t = grp; t < nmine; t += kGroups) {
            const int s = t % kNst, b = t % kNTile, kk = t / kGroups;
            if (!wait(&st_full[s], (uint32_t)((t / kNst) & 1))) break;
            if (t >= kNTile && !wait(&tl_empty[b], (uint32_t)((t / kNTile - 1) & 1))) break;
            const float *U = reinterpret_cast<const float *>(stg + s * kStage);
            const double *Pe = reinterpret_cast<const double *>(stg + s * kStage + kStK);
            unsigned char *Ab = A + b * kBufA, *Bb = B + b * kBufB;
            float *ps = psum + (grp * 2 + (kk & 1)) * (8 * KR * 3);
            float hi[8], lo[8];
            if (b_task) {
                // P_e(c, j) at c*16 + j: FP32 high and low parts, and this
                // segment's sums by direction for the case's mean translation
#pragma unroll
                for (int g = 0; g < 8; ++g) {
                    const int c = 8 * qb + g;
                    split_f64(c < 60 ? Pe[c * KR + j] : 0.0, hi[g], lo[g]);
                }
                const float u0 = hi[0] + hi[3] + hi[6], u1 = hi[1] + hi[4] + hi[7], u2 = hi[2] + hi[5];
                ps[(qb * KR + j) * 3 + 0] = rb == 0 ? u0 : rb == 1 ? u2 : u1;
                ps[(qb * KR + j) * 3 + 1] = rb == 0 ? u1 : rb == 1 ? u0 : u2;
                ps[(qb * KR + j) * 3 + 2] = rb == 0 ? u2 : rb == 1 ? u1 : u0;
                __syncwarp();
                if (lane == 0) mbar_arrive(my_sum);
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (a_task[h]) {
                    float xv[8];
#pragma unroll
                    for (int g = 0; g < 8; ++g) xv[g] = U[off[h][g]];
                    split3_store8(xv, Ab + a_off[h], kTermA);
                }
            }
            if (b_task) {
                // the four B warps' partial sums are in (bounded wait; the
                // double buffer is safe because no warp of the group passes
                // the wait for its next element before every one of them has
                // arrived for it)
                if (!wait(my_sum, (uint32_t)(kk & 1))) break;
                float tdir[3];
#pragma unroll
                for (int dd = 0; dd < 3; ++dd) {
                    float acc = 0.f;
#pragma unroll
                    for (int c8 = 0; c8 < 8; ++c8) acc += ps[(c8 * KR + j) * 3 + dd];
                    tdir[dd] = 0.05f * acc;
                }
                const float t0 = tdir[0], t1 = tdir[1], t2 = tdir[2];
                const float tr[3] = {rb == 0 ? t0 : rb == 1 ? t1 : t2, rb == 0 ? t1 : rb == 1 ? t2 : t0,
                                     rb == 0 ? t2 : rb == 1 ? t0 : t1};
                float xv[8];
#pragma unroll
                for (int g = 0; g < 8; ++g) xv[g] = (8 * qb + g < 60) ? (hi[g] - tr[g % 3]) + lo[g] : 0.f;
                split3_store8(xv, Bb + kmajor_off(j, 8 * qb), kTermB);
            }
            fence_proxy_async();   // this thread's tile writes -> the tensor cores
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&st_empty[s]);
                mbar_arrive(&tl_full[b]);
            }
        }
    } else if (warp == kMmaWarp) {
        int t = 0;
        if (lane == 0) {
            for (; t < nmine; ++t) {
                const int b = t % kNTile, a = t % kNAcc;
                if (!wait(&tl_full[b], (uint32_t)((t / kNTile) & 1))) break;
                if (t >= kNAcc && !wait(&ac_empty[a], (uint32_t)((t / kNAcc - 1) & 1))) break;
                tc_fence_after();
                const uint32_t a0 = smem_u32(A + b * kBufA), b0 = smem_u32(B + b * kBufB);
                // the six products of order <= 2^-16: (1,1) (1,2) (2,1) (1,3) (2,2) (3,1)
                const int ta[6] = {0, 0, 1, 0, 1, 2};
                const int tb[6] = {0, 1, 0, 2, 1, 0};
                uint32_t acc = 0;
#pragma unroll
                for (int tt = 0; tt < 6; ++tt)
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks) {   // K = 64 in steps of 16 (two core matrices)
                        mma_bf16(tmem + (uint32_t)(16 * a), umma_desc(a0 + ta[tt] * kTermA + ks * 256, 128, 1024),
                                 umma_desc(b0 + tb[tt] * kTermB + ks * 256, 128, 1024), kIdesc, acc);
                        acc = 1;
                    }
                mma_commit(&tl_empty[b]);
                mma_commit(&ac_full[a]);
            }
            s_count[1] = t;
        }
        __syncwarp();
    } else if (warp >= kEpiWarp0 && warp < kEpiWarp0 + kNEpi) {
        // direction dn: TMEM lane i < 20 holds row 3i + dn for the 16 cases,
        // lane 20 the sum of those rows; subtracting a twentieth of it
        // removes each case's mean translation from the result
        const int dn = warp - kEpiWarp0;
        for (int t = 0; t < nmine; ++t) {
            const int a = t % kNAcc;
            if (!wait(&ac_full[a], (uint32_t)((t / kNAcc) & 1))) break;
            tc_fence_after();
            float v[16];
            tmem_ld_32x32b_x16(tmem + ((uint32_t)(32 * dn) << 16) + (uint32_t)(16 * a), v);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ac_empty[a]);
#pragma unroll
            for (int x = 0; x < 16; ++x) v[x] -= 0.05f * __shfl_sync(kFullMask, v[x], 20);
            if (lane < 20) {
                float4 *o = reinterpret_cast<float4 *>(ut + ((size_t)elem(t) * 60 + 3 * lane + dn) * KR);
                o[0] = make_float4(v[0], v[1], v[2], v[3]);
                o[1] = make_float4(v[4], v[5], v[6], v[7]);
                o[2] = make_float4(v[8], v[9], v[10], v[11]);
                o[3] = make_float4(v[12], v[13], v[14], v[15]);
            }
        }
    }
    __syncthreads();
    if (*s_fail) {
        if (tid == 0) {
            atomicExch(err, 3);
            // copies issued: elements 0 .. s_count[0]-1; MMA groups committed: 0 .. s_count[1]-1.
            // Wait (bounded) for the last phase of every stage and accumulator still owed.
            for (int t = s_count[0] - kNst; t < s_count[0]; ++t)
                if (t >= 0) mbar_wait(&st_full[t % kNst], (uint32_t)((t / kNst) & 1));
            for (int t = s_count[1] - kNAcc; t < s_count[1]; ++t)
                if (t >= 0) mbar_wait(&ac_full[t % kNAcc], (uint32_t)((t / kNAcc) & 1));
        }
        __syncthreads();
    }
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 64);
}

// Block element products on CUDA cores (FP32 or FP64): one warp per element,
// lanes own rows 2l, 2l+1; P_e staged in shared memory per warp.
template <typename KT, typename OT>
__global__ void __launch_bounds__(256)
k_mr_elem_cc(int nels, const KT *__restrict__ km, const int *__restrict__ conn, const double *__restrict__ P,
             OT *__restrict__ ut, const int *__restrict__ skip)
{
    constexpr int WPB = 32 / (int)sizeof(KT);   // warps per block: 8 (FP32) or 4 (FP64), 30 KB of P blocks
    __shared__ KT ps[WPB][60 * KR];
    if (skip && *skip) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int e = warp; e < nels; e += nwarps) {
        for (int idx = lane; idx < 60 * KR; idx += 32) {
            const int c = idx / KR, j = idx - KR * c;
            const int nd = conn[(size_t)e * 20 + c / 3];
            ps[w][idx] = (KT)P[((size_t)3 * nd + c % 3) * KR + j];
        }
        __syncwarp();
        if (lane < 30) {
            KT a0[KR], a1[KR];
#pragma unroll
            for (int j = 0; j < KR; ++j) a0[j] = a1[j] = (KT)0;
            const KT *ke = km + (size_t)e * 3600 + 2 * lane;
            for (int c = 0; c < 60; ++c) {
                const KT k0 = ke[60 * c], k1 = ke[60 * c + 1];
#pragma unroll
                for (int j = 0; j < KR; ++j) {
                    const KT pj = ps[w][c * KR + j];
                    a0[j] = fma(k0, pj, a0[j]);
                    a1[j] = fma(k1, pj, a1[j]);
                }
            }
            OT *o0 = ut + ((size_t)e * 60 + 2 * lane) * KR;
#pragma unroll
            for (int j = 0; j < KR; ++j) {
                o0[j] = (OT)a0[j];
                o0[KR + j] = (OT)a1[j];
            }
        }
        __syncwarp();
    }
}

// Node scatter for k load cases: thread (node, j), ascending element order.
// MODE 0: U = sum, partial p.u per case; MODE 1: RRES = F - sum, partial rr.
template <typename UT, int MODE>
__global__ void __launch_bounds__(256)
k_mr_scatter(int nn, const int *__restrict__ ptr, const int *__restrict__ list, const UT *__restrict__ ut,
             const uint8_t *__restrict__ fm, const double *__restrict__ pf, double *__restrict__ out,
             double *__restrict__ part, const int *__restrict__ skip)
{
    if (skip && *skip) return;   // uniform: the flag does not change during the kernel
    const int j = threadIdx.x & (KR - 1);
    double loc = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nn * KR; t += gridDim.x * blockDim.x) {
        const int n = t / KR;
        UT a0 = 0, a1 = 0, a2 = 0;   // FP32 products are summed in FP32, FP64 ones in FP64
        for (int k = ptr[n]; k < ptr[n + 1]; ++k) {
            const size_t base = (size_t)list[k] * 3 * KR + j;   // list holds e*20+a
            a0 += ut[base];
            a1 += ut[base + KR];
            a2 += ut[base + 2 * KR];
        }
        const int m = fm[n];
        const double a[3] = {(double)a0, (double)a1, (double)a2};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const size_t s = ((size_t)3 * n + d) * KR + j;
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
    }
    // per-case block reduction: lanes l and l+16 share a case
    loc += __shfl_xor_sync(kFullMask, loc, 16);
    __shared__ double sh[8][KR];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane < KR) sh[w][lane] = loc;
    __syncthreads();
    if (threadIdx.x < KR) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i][threadIdx.x];
        part[(size_t)blockIdx.x * KR + threadIdx.x] = s;
    }
}

// per-case state
struct MState {
    double up[KR], ff[KR], rr[KR], thr[KR];
    double alpha[KR], beta[KR];   // this iteration's step lengths (0 for inactive cases)
    int active[KR];      // 1 until the case's true residual reaches tol
    int flag[KR];        // recursive residual reached thr (replacement wanted)
    int iters[KR];
    int any_flag;        // stop iterating: some active case wants a replacement
    int pending;         // set by this iteration's k_mr_beta, moved to any_flag by k_mr_finish
    int err;
};

// per-case sums of block partials (fixed order, same value in every block)
__device__ __forceinline__ double case_sum(const double *part, int G, int j)
{
    double s = 0.0;
    for (int b = 0; b < G; ++b) s += part[(size_t)b * KR + j];
    return s;
}

// The same sums by one 256-thread block: thread (g, j) adds partials
// g, g+16, ... of case j, then thread j adds the 16 group sums in order.
// Fixed order, so the result is the same in every run.
__device__ __forceinline__ double case_sum_block(const double *part, int G, double (*sh)[KR])
{
    const int j = threadIdx.x & (KR - 1), g = threadIdx.x >> 4;
    double s = 0.0;
    for (int b = g; b < G; b += 16) s += part[(size_t)b * KR + j];
    sh[g][j] = s;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < KR)
        for (int i = 0; i < 16; ++i) t += sh[i][threadIdx.x];
    __syncthreads();
    return t;   // valid in threads 0..15
}

template <int NV>
__device__ __forceinline__ void case_block_reduce(double (&v)[NV], unsigned kinds, double *out, size_t stride)
{
    // lanes l and l+16 hold the same case
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const double o = __shfl_xor_sync(kFullMask, v[k], 16);
        v[k] = ((kinds >> k) & 1) ? fmax(v[k], o) : v[k] + o;
    }
    __shared__ double sh[NV][8][KR];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane < KR)
#pragma unroll
        for (int k = 0; k < NV; ++k) sh[k][w][lane] = v[k];
    __syncthreads();
    if (threadIdx.x < KR)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = 0.0;
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i)
                s = ((kinds >> k) & 1) ? fmax(s, sh[k][i][threadIdx.x]) : s + sh[k][i][threadIdx.x];
            out[k * stride + (size_t)blockIdx.x * KR + threadIdx.x] = s;
        }
}

__global__ void __launch_bounds__(256)
k_mr_init(int ns, const double *__restrict__ F, const double *__restrict__ dinv, double *__restrict__ X,
          double *__restrict__ R, double *__restrict__ D, double *__restrict__ P, double *__restrict__ part, int G)
{
    double rd = 0.0, rr = 0.0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)ns * KR;
         t += (size_t)gridDim.x * blockDim.x) {
        const double rv = F[t], dv = dinv[t / KR] * rv;
        X[t] = 0.0;
        R[t] = rv;
        D[t] = dv;
        P[t] = dv;
        rd = fma(rv, dv, rd);
        rr = fma(rv, rv, rr);
    }
    double v[2] = {rd, rr};
    case_block_reduce<2>(v, 0u, part, (size_t)G * KR);
}

__global__ void k_mr_init2(MState *st, const double *__restrict__ part, int G, double tol)
{
    const int j = threadIdx.x;
    if (j >= KR) return;
    const double rd = case_sum(part, G, j), rr = case_sum(part + (size_t)G * KR, G, j);
    st->up[j] = rd;
    st->ff[j] = rr;
    st->rr[j] = rr;
    st->thr[j] = 0.1 > tol ? 0.1 : tol;
    st->active[j] = rr > 0.0 ? 1 : 0;
    st->flag[j] = 0;
    st->iters[j] = 0;
    if (j == 0) {
        st->any_flag = 0;
        st->pending = 0;
        st->err = 0;
    }
}

// alpha = up / (p.u) per case, from the scatter's partials (one block)
__global__ void __launch_bounds__(256) k_mr_alpha(MState *st, const double *__restrict__ ps, int Gs)
{
    __shared__ double sh[16][KR];
    if (st->any_flag) return;
    const double pu = case_sum_block(ps, Gs, sh);
    const int j = threadIdx.x;
    if (j < KR) st->alpha[j] = st->active[j] ? st->up[j] / pu : 0.0;
}

__global__ void __launch_bounds__(256)
k_mr_update1(int ns, const MState *__restrict__ st, double *__restrict__ pu_out, int G, double *__restrict__ X,
             double *__restrict__ R, double *__restrict__ D, const double *__restrict__ P,
             const double *__restrict__ U, const double *__restrict__ dinv)
{
    if (st->any_flag) return;
    const int j = threadIdx.x & (KR - 1);
    const double alpha = st->alpha[j];
    double rd = 0.0, rr = 0.0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)ns * KR;
         t += (size_t)gridDim.x * blockDim.x) {
        X[t] = fma(P[t], alpha, X[t]);
        const double rn = fma(-U[t], alpha, R[t]);
        R[t] = rn;
        const double dn = dinv[t / KR] * rn;
        D[t] = dn;
        rd = fma(rn, dn, rd);
        rr = fma(rn, rn, rr);
    }
    double v[2] = {rd, rr};
    case_block_reduce<2>(v, 0u, pu_out, (size_t)G * KR);
}

// r.d and r.r per case; beta = (r.d)_new / up; the new up, rr and iteration
// count; the stopping test (one block).  The flag raised here reaches
// any_flag only in k_mr_finish, after this iteration's k_mr_update2.
__global__ void __launch_bounds__(256) k_mr_beta(MState *st, const double *__restrict__ part, int G, int limit)
{
    __shared__ double sh[16][KR];
    __shared__ int s_any;
    if (st->any_flag) return;
    if (threadIdx.x == 0) s_any = 0;
    const double rd = case_sum_block(part, G, sh);
    const double rr = case_sum_block(part + (size_t)G * KR, G, sh);
    const int j = threadIdx.x;
    if (j < KR) {
        if (st->active[j]) {
            st->beta[j] = rd / st->up[j];
            st->up[j] = rd;
            st->rr[j] = rr;
            st->iters[j] += 1;
            const bool f = sqrt(rr) / sqrt(st->ff[j]) <= st->thr[j] || st->iters[j] >= limit || !isfinite(rd);
            st->flag[j] = f ? 1 : 0;
            if (!isfinite(rd)) st->err = 1;
            if (f) atomicOr(&s_any, 1);
        } else {
            st->beta[j] = 0.0;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_any) st->pending = 1;
}

__global__ void __launch_bounds__(256)
k_mr_update2(int ns, const MState *__restrict__ st, const double *__restrict__ D, double *__restrict__ P)
{
    if (st->any_flag) return;
    const int j = threadIdx.x & (KR - 1);
    const double beta = st->beta[j];
    const bool act = st->active[j] != 0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)ns * KR;
         t += (size_t)gridDim.x * blockDim.x)
        if (act) P[t] = fma(P[t], beta, D[t]);
}

__global__ void k_mr_finish(MState *st)
{
    if (threadIdx.x == 0 && !st->any_flag && st->pending) {
        st->any_flag = 1;
        st->pending = 0;
    }
}

// residual replacement: R = RRES for active cases, D = dinv*R, partials r.d, r.r
__global__ void __launch_bounds__(256)
k_mr_replace(int ns, const MState *__restrict__ st, const double *__restrict__ RRES,
             const double *__restrict__ dinv, double *__restrict__ R, double *__restrict__ D,
             double *__restrict__ part, int G)
{
    const int j = threadIdx.x & (KR - 1);
    double rd = 0.0, rr = 0.0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)ns * KR;
         t += (size_t)gridDim.x * blockDim.x) {
        if (!st->active[j]) continue;
        const double rv = RRES[t], dv = dinv[t / KR] * rv;
        R[t] = rv;
        D[t] = dv;
        rd = fma(rv, dv, rd);
        rr = fma(rv, rv, rr);
    }
    double v[2] = {rd, rr};
    case_block_reduce<2>(v, 0u, part, (size_t)G * KR);
}

__global__ void k_mr_replace2(MState *st, const double *__restrict__ part, int G)
{
    const int j = threadIdx.x;
    if (j < KR && st->active[j]) {
        st->up[j] = case_sum(part, G, j);
        st->rr[j] = case_sum(part + (size_t)G * KR, G, j);
        st->flag[j] = 0;
    }
    if (j == 0) {
        st->any_flag = 0;
        st->pending = 0;
    }
}

// ksum[e][d][k] = sum over the 20 nodes a of K_e(3a + d, k) from the packed
// FP32 storkm (summed in FP64), 0 for k = 60..63: the direction sums of
// K_e's rows that the tensor-core block product adds to its A operand.
__global__ void k_mr_rowsums(int nels, const float *__restrict__ kp, float *__restrict__ ksum)
{
    const size_t total = (size_t)nels * 192;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const size_t e = idx / 192;
        const int r = (int)(idx - e * 192), d = r / 64, k = r % 64;
        float v = 0.f;
        if (k < 60) {
            const float *ke = kp + e * 1832;
            double sum = 0.0;
            for (int a = 0; a < 20; ++a) sum += (double)ke[packed_off(3 * a + d, k)];
            v = (float)sum;
        }
        ksum[idx] = v;
    }
}

__global__ void k_mr_sums(const double *__restrict__ part, int G, double *__restrict__ out)
{
    if (threadIdx.x < KR) out[threadIdx.x] = case_sum(part, G, threadIdx.x);
}

__global__ void k_mr_eq_to_slot(int ns, const int *__restrict__ slot_eq, int neq, const double *__restrict__ Req,
                                double *__restrict__ F)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)ns * KR;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t s = t / KR, j = t % KR;
        const int q = slot_eq[s];
        F[t] = q > 0 ? Req[j * (size_t)neq + q - 1] : 0.0;
    }
}

__global__ void k_mr_slot_to_eq(int neq, const int *__restrict__ eq_slot, const double *__restrict__ X,
                                double *__restrict__ Xeq)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)neq * KR;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t j = t / neq, q = t % neq;
        Xeq[t] = X[(size_t)eq_slot[q] * KR + j];
    }
}

// ---------------------------------------------------------------------------
// Block-solve buffers of one context (Ctx::multi), allocated on the first
// block solve or product and kept while the mesh is unchanged.
struct MultiBufs {
    int ns = 0;
    double *F = nullptr, *X = nullptr, *R = nullptr, *D = nullptr, *P = nullptr, *U = nullptr, *RR = nullptr,
           *eq = nullptr;
    int ne = 0;
    float *ut32 = nullptr;
    float *ksum = nullptr;   // [nels][3][64] direction sums of K_e's rows (tensor-core products)
    double *ut64 = nullptr, *part = nullptr, *sums = nullptr;
    MState *st = nullptr;
    MState *hst = nullptr;
};
namespace {
void mb_free(MultiBufs &m)
{
    void *p[] = {m.F, m.X, m.R, m.D, m.P, m.U, m.RR, m.eq, m.ut32, m.ksum, m.ut64, m.part, m.sums, m.st};
    for (void *q : p)
        if (q) cudaFree(q);
    if (m.hst) cudaFreeHost(m.hst);
    m = MultiBufs();
}
}  // namespace

void multi_release(Ctx &c)
{
    if (!c.multi) return;
    mb_free(*c.multi);
    delete c.multi;
    c.multi = nullptr;
}

}  // namespace pf

using namespace pf;

#define MCK(call)                                                                        \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return PF_FAILURE;                                                           \
        }                                                                                \
    } while (0)

static int mr_launched(Ctx &c, const char *name)
{
    c.launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: launch failed: %s", name, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

// U = K P for the block (prec 16: tensor cores, 32: CUDA-core FP32, 64: FP64
// into ut64).  skip: device flag that turns the launch into a no-op.
static int mr_elem(Ctx &c, int prec, const double *P, const int *skip)
{
    MultiBufs &m = *c.multi;
    if (prec == 16) {
        const int smem = kTcSmem;
        MCK(cudaFuncSetAttribute(k_mr_elem_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        const int grid = c.nels < c.nsm ? c.nels : c.nsm;
        k_mr_elem_tc<<<grid, kTcThreads, smem, c.stream>>>(c.nels, c.km32p, m.ksum, c.conn, P, m.ut32, c.kerr, skip);
        return mr_launched(c, "k_mr_elem_tc");
    }
    if (prec == 32) {
        const int grid = (c.nels + 7) / 8 < c.nsm * 8 ? (c.nels + 7) / 8 : c.nsm * 8;
        k_mr_elem_cc<float, float><<<grid, 256, 0, c.stream>>>(c.nels, c.km32, c.conn, P, m.ut32, skip);
        return mr_launched(c, "k_mr_elem_cc<float>");
    }
    const int grid = (c.nels + 3) / 4 < c.nsm * 16 ? (c.nels + 3) / 4 : c.nsm * 16;
    k_mr_elem_cc<double, double><<<grid, 128, 0, c.stream>>>(c.nels, c.km64, c.conn, P, m.ut64, skip);
    return mr_launched(c, "k_mr_elem_cc<double>");
}

static int mr_scatter(Ctx &c, int prec, int mode, const double *pf, double *out, const int *skip)
{
    MultiBufs &m = *c.multi;
    const int G = c.Gs;
    if (prec == 64) {
        if (mode == 0) k_mr_scatter<double, 0><<<G, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, m.ut64, c.freemask, pf, out, m.part, skip);
        else k_mr_scatter<double, 1><<<G, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, m.ut64, c.freemask, pf, out, m.part, skip);
    } else {
        if (mode == 0) k_mr_scatter<float, 0><<<G, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, m.ut32, c.freemask, pf, out, m.part, skip);
        else k_mr_scatter<float, 1><<<G, 256, 0, c.stream>>>(c.nn, c.node_ptr, c.node_list, m.ut32, c.freemask, pf, out, m.part, skip);
    }
    return mr_launched(c, "k_mr_scatter");
}

static int mr_alloc(Ctx &c)
{
    if (!c.multi) c.multi = new MultiBufs();
    MultiBufs &m = *c.multi;
    if (m.ns == c.nslots && m.ne == c.nels && m.F) return 0;
    mb_free(m);
    const size_t n = (size_t)c.nslots * KR;
    const size_t parts = (size_t)(c.Gs > c.G ? c.Gs : c.G) * KR * 4 + 64;
    double **v[] = {&m.F, &m.X, &m.R, &m.D, &m.P, &m.U, &m.RR};
    for (double **q : v)
        if (cudaMalloc((void **)q, n * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.eq, (size_t)(c.neq > 0 ? c.neq : 1) * KR * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.ut32, (size_t)c.nels * 60 * KR * 4) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.ksum, (size_t)c.nels * 192 * 4) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.ut64, (size_t)c.nels * 60 * KR * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.part, parts * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.sums, 64 * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.st, sizeof(MState)) != cudaSuccess) goto fail;
    if (cudaMallocHost((void **)&m.hst, sizeof(MState)) != cudaSuccess) goto fail;
    m.ns = c.nslots;
    m.ne = c.nels;
    return 0;
fail:
    mb_free(m);
    set_error("pf_solve_multi: cannot allocate the block vectors (%zu slots x %d cases)", (size_t)c.nslots, KR);
    return 1;
}

// direction sums of the packed storkm's rows for the tensor-core block
// product (once per solve or product call: storkm may have changed)
static int mr_rowsums(Ctx &c)
{
    const int grid = c.nsm * 8;
    k_mr_rowsums<<<grid, 256, 0, c.stream>>>(c.nels, c.km32p, c.multi->ksum);
    return mr_launched(c, "k_mr_rowsums");
}

// FP64 true residuals of all cases; returns per-case ||f - K x||^2 in rr_out
static int mr_true_residual(Ctx &c, double *rr_out)
{
    MultiBufs &m = *c.multi;
    if (mr_elem(c, 64, m.X, nullptr)) return 1;
    if (mr_scatter(c, 64, 1, m.F, m.RR, nullptr)) return 1;
    k_mr_sums<<<1, 32, 0, c.stream>>>(m.part, c.Gs, m.sums);
    if (mr_launched(c, "k_mr_sums")) return 1;
    MCK(cudaMemcpyAsync(rr_out, m.sums, KR * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    MCK(cudaStreamSynchronize(c.stream));
    return 0;
}

extern "C" int pf_solve_multi(void **ctx, const int *k, const double *r, const double *tol, const int *limit,
                              const int *prec, double *xnew, int *iters, double *relres)
{
    if (!ctx || !*ctx || !k || !r || !tol || !limit || !prec || !xnew || !iters || !relres) {
        set_error("pf_solve_multi: null argument");
        return PF_FAILURE;
    }
    Ctx &c = *(Ctx *)*ctx;
    MCK(cudaSetDevice(c.device));
    if (*k != KR) {
        set_error("pf_solve_multi: k must be %d", KR);
        return PF_FAILURE;
    }
    if (c.shared || c.kind != KIND_SOLID20) {
        set_error("pf_solve_multi: needs per-element 20-node storkm");
        return PF_FAILURE;
    }
    if (!c.have_km || *limit < 1 || (*prec != 16 && *prec != 32)) {
        set_error("pf_solve_multi: needs storkm, limit >= 1 and prec 16 (tensor cores) or 32 (CUDA cores)");
        return PF_FAILURE;
    }
    if (mr_alloc(c)) return PF_FAILURE;
    if (*prec == 16 && mr_rowsums(c)) return PF_FAILURE;
    MultiBufs &m = *c.multi;
    const int G = c.G, Gs = c.Gs;
    // load cases: r(neq, k) column-major
    MCK(cudaMemcpyAsync(m.eq, r, (size_t)c.neq * KR * 8, cudaMemcpyHostToDevice, c.stream));
    k_mr_eq_to_slot<<<c.nsm * 8, 256, 0, c.stream>>>(c.nslots, c.slot_eq, c.neq, m.eq, m.F);
    if (mr_launched(c, "k_mr_eq_to_slot")) return PF_FAILURE;
    cudaEvent_t e0, e1;
    MCK(cudaEventCreate(&e0));
    MCK(cudaEventCreate(&e1));
    MCK(cudaEventRecord(e0, c.stream));
    k_mr_init<<<G, 256, 0, c.stream>>>(c.nslots, m.F, c.dinv, m.X, m.R, m.D, m.P, m.part, G);
    if (mr_launched(c, "k_mr_init")) return PF_FAILURE;
    k_mr_init2<<<1, 32, 0, c.stream>>>(m.st, m.part, G, *tol);
    if (mr_launched(c, "k_mr_init2")) return PF_FAILURE;
    double *pu = m.part + (size_t)Gs * KR;   // update partials after the scatter partials
    int total = 0, chunk = 4, corrections = 0;
    double rel[KR] = {0};
    // per-kernel timing of the iterations: events around the element product
    // and the scatter of every launched iteration (pool reused per chunk)
    constexpr int kMaxChunk = 32;
    cudaEvent_t tev[3 * kMaxChunk];
    for (auto &ev : tev) MCK(cudaEventCreate(&ev));
    double ms_elem = 0.0, ms_scat = 0.0, ms_iter = 0.0;
    for (;;) {
        for (int i = 0; i < chunk; ++i) {
            const int *skip = &m.st->any_flag;
            MCK(cudaEventRecord(tev[3 * i], c.stream));
            if (mr_elem(c, *prec, m.P, skip)) return PF_FAILURE;
            MCK(cudaEventRecord(tev[3 * i + 1], c.stream));
            if (mr_scatter(c, *prec, 0, m.P, m.U, skip)) return PF_FAILURE;
            MCK(cudaEventRecord(tev[3 * i + 2], c.stream));
            k_mr_alpha<<<1, 256, 0, c.stream>>>(m.st, m.part, Gs);
            if (mr_launched(c, "k_mr_alpha")) return PF_FAILURE;
            k_mr_update1<<<G, 256, 0, c.stream>>>(c.nslots, m.st, pu, G, m.X, m.R, m.D, m.P, m.U, c.dinv);
            if (mr_launched(c, "k_mr_update1")) return PF_FAILURE;
            k_mr_beta<<<1, 256, 0, c.stream>>>(m.st, pu, G, *limit);
            if (mr_launched(c, "k_mr_beta")) return PF_FAILURE;
            k_mr_update2<<<G, 256, 0, c.stream>>>(c.nslots, m.st, m.D, m.P);
            if (mr_launched(c, "k_mr_update2")) return PF_FAILURE;
            k_mr_finish<<<1, 32, 0, c.stream>>>(m.st);
            if (mr_launched(c, "k_mr_finish")) return PF_FAILURE;
        }
        total += chunk;
        MCK(cudaMemcpyAsync(m.hst, m.st, sizeof(MState), cudaMemcpyDeviceToHost, c.stream));
        MCK(cudaStreamSynchronize(c.stream));
        for (int i = 0; i < chunk; ++i) {
            float a = 0.f, b = 0.f, d = 0.f;
            cudaEventElapsedTime(&a, tev[3 * i], tev[3 * i + 1]);
            cudaEventElapsedTime(&b, tev[3 * i + 1], tev[3 * i + 2]);
            if (i + 1 < chunk) cudaEventElapsedTime(&d, tev[3 * i], tev[3 * i + 3]);
            ms_elem += a;
            ms_scat += b;
            ms_iter += d;
        }
        if (chunk < kMaxChunk) chunk *= 2;
        int kerr = 0;
        MCK(cudaMemcpy(&kerr, c.kerr, sizeof(int), cudaMemcpyDeviceToHost));
        if (kerr) {
            cudaMemset(c.kerr, 0, sizeof(int));
            set_error("pf_solve_multi: tensor-core product wait timed out");
            return PF_FAILURE;
        }
        if (m.hst->err) {
            set_error("pf_solve_multi: PCG breakdown (non-finite r.d)");
            return PF_FAILURE;
        }
        if (!m.hst->any_flag) continue;
        // some active case reached its threshold (or the limit): FP64 true residuals
        double rr[KR];
        if (mr_true_residual(c, rr)) return PF_FAILURE;
        int n_active = 0;
        for (int j = 0; j < KR; ++j) {
            rel[j] = m.hst->ff[j] > 0 ? std::sqrt(rr[j]) / std::sqrt(m.hst->ff[j]) : 0.0;
            if (m.hst->active[j]) {
                if (rel[j] <= *tol || m.hst->iters[j] >= *limit) m.hst->active[j] = 0;
                else {
                    m.hst->thr[j] = 0.1 * rel[j] > *tol ? 0.1 * rel[j] : 0.5 * *tol;
                    ++n_active;
                }
            }
        }
        if (n_active == 0) break;
        // push the new thresholds and active flags, then replace the residuals
        MCK(cudaMemcpyAsync(m.st, m.hst, sizeof(MState), cudaMemcpyHostToDevice, c.stream));
        k_mr_replace<<<G, 256, 0, c.stream>>>(c.nslots, m.st, m.RR, c.dinv, m.R, m.D, m.part, G);
        if (mr_launched(c, "k_mr_replace")) return PF_FAILURE;
        k_mr_replace2<<<1, 32, 0, c.stream>>>(m.st, m.part, G);
        if (mr_launched(c, "k_mr_replace2")) return PF_FAILURE;
        ++corrections;
        chunk = 4;
    }
    for (auto &ev : tev) cudaEventDestroy(ev);
    MCK(cudaEventRecord(e1, c.stream));
    k_mr_slot_to_eq<<<c.nsm * 8, 256, 0, c.stream>>>(c.neq, c.eq_slot, m.X, m.eq);
    if (mr_launched(c, "k_mr_slot_to_eq")) return PF_FAILURE;
    MCK(cudaMemcpyAsync(xnew, m.eq, (size_t)c.neq * KR * 8, cudaMemcpyDeviceToHost, c.stream));
    MCK(cudaStreamSynchronize(c.stream));
    float ms = 0.f;
    MCK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int j = 0; j < KR; ++j) {
        iters[j] = m.hst->iters[j];
        relres[j] = rel[j];
    }
    c.stats[0] = 0;
    for (int j = 0; j < KR; ++j) c.stats[0] = iters[j] > c.stats[0] ? iters[j] : c.stats[0];
    c.stats[1] = corrections;
    c.stats[2] = ms;
    c.stats[3] = ms_elem;   // summed element-product time of the launched iterations
    c.stats[4] = ms_scat;   // summed scatter time
    c.stats[5] = ms_iter;   // summed time of the iterations measured start to start
    c.stats[6] = total;     // iterations launched (including no-op ones after a flag)
    return PF_SUCCESS;
}

// Block product U = K P for k = 16 cases in equation order (tests): prec 16,
// 32 or 64.
extern "C" int pf_ebe_matvec_multi(void **ctx, const int *k, const int *prec, const double *p, double *u)
{
    if (!ctx || !*ctx || !k || !prec || !p || !u) {
        set_error("pf_ebe_matvec_multi: null argument");
        return PF_FAILURE;
    }
    Ctx &c = *(Ctx *)*ctx;
    MCK(cudaSetDevice(c.device));
    if (*k != KR || !c.have_km || c.shared || c.kind != KIND_SOLID20 || (*prec != 16 && *prec != 32 && *prec != 64)) {
        set_error("pf_ebe_matvec_multi: k must be %d, prec 16/32/64, per-element storkm formed", KR);
        return PF_FAILURE;
    }
    if (mr_alloc(c)) return PF_FAILURE;
    if (*prec == 16 && mr_rowsums(c)) return PF_FAILURE;
    MultiBufs &m = *c.multi;
    MCK(cudaMemcpyAsync(m.eq, p, (size_t)c.neq * KR * 8, cudaMemcpyHostToDevice, c.stream));
    k_mr_eq_to_slot<<<c.nsm * 8, 256, 0, c.stream>>>(c.nslots, c.slot_eq, c.neq, m.eq, m.P);
    if (mr_launched(c, "k_mr_eq_to_slot")) return PF_FAILURE;
    if (mr_elem(c, *prec, m.P, nullptr)) return PF_FAILURE;
    if (mr_scatter(c, *prec, 0, m.P, m.U, nullptr)) return PF_FAILURE;
    k_mr_slot_to_eq<<<c.nsm * 8, 256, 0, c.stream>>>(c.neq, c.eq_slot, m.U, m.eq);
    if (mr_launched(c, "k_mr_slot_to_eq")) return PF_FAILURE;
    MCK(cudaMemcpyAsync(u, m.eq, (size_t)c.neq * KR * 8, cudaMemcpyDeviceToHost, c.stream));
    MCK(cudaStreamSynchronize(c.stream));
    int kerr = 0;
    MCK(cudaMemcpy(&kerr, c.kerr, sizeof(int), cudaMemcpyDeviceToHost));
    if (kerr) {
        cudaMemset(c.kerr, 0, sizeof(int));
        set_error("pf_ebe_matvec_multi: tensor-core product wait timed out");
        return PF_FAILURE;
    }
    return PF_SUCCESS;
}

extern "C" int pf_multi_free(void **ctx)
{
    if (!ctx || !*ctx) return PF_SUCCESS;
    Ctx &c = *(Ctx *)*ctx;
    cudaSetDevice(c.device);
    cudaStreamSynchronize(c.stream);
    multi_release(c);
    return PF_SUCCESS;
}
