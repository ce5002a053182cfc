// pf_multi.cu -- k load cases of one mesh solved together (block PCG).
//
// k independent Jacobi-PCG solves (p121.f90:86-104) share every element
// matrix read: one iteration computes U = K P for a 60 x k block per element.
// Vectors are interleaved per slot, v[slot*k + j], so the gather of an
// element's block and the node scatter touch k consecutive values.  k is
// any multiple of 8 up to kMaxK.
//
// Element products:
//   k_mr_elem_h16  tensor cores (tcgen05.mma, kind::f16, FP16 operands, FP32
//                  accumulation in TMEM).  K_e is split once, when storkm is
//                  formed or set, into two FP16 terms (hi + lo, about 22
//                  significant bits, scaled per element by a power of two)
//                  stored in the tensor cores' shared-memory tile layout;
//                  P_e less a translation of each case is split the same way
//                  per element and case.  The four products of the two
//                  splits are summed: the block product reaches FP32-class
//                  accuracy.  Cases are taken in
//                  passes of 64, 32, 16 or 8 (the MMA's N is twice that),
//                  the widest pass chosen by timing on the mesh.
//   k_mr_elem_cc   the same product on CUDA cores in FP32 (check kernel for
//                  the tensor-core one, selectable by prec) and in FP64
//                  (DFMA) for the true residual f - K x.
// The inner PCG runs on the FP32-class product with FP64 vectors, dots and
// alpha/beta; the recursive residuals are replaced by the FP64 true residual
// whenever an active load case has dropped 10x (as PF_MODE_MIXED does).
#include "pf_device.cuh"
#include "pf_tc.cuh"
#include "pfgpu.h"

#include <cstring>
#include <cuda.h>   // CUtensorMap (the encoder is reached through the runtime's driver entry point)
#include <cuda_fp16.h>
#include <vector>

namespace pf {

using namespace tc;

namespace {

constexpr int kMaxK = 128;           // load cases of one block solve
constexpr int kMaxKB = 64;           // cases of one tensor-core pass (the MMA's N)
constexpr unsigned kFullMask = 0xffffffffu;

// ---- the stored element record of the tensor-core product -----------------
// A tile (M = 128 rows, K = 64 columns, FP16, K-major, no swizzle): 16 x 8
// core matrices of 8 rows x 16 bytes, core matrix (I, J) at 1024 I + 128 J
// (SBO = 1024 B between row groups, LBO = 128 B between column groups).
// Rows 0..63 hold the high FP16 term of K_e, rows 64..127 the low term.
// Within a term, rows and columns are ordered by direction: row (column)
// 20 d + i is dof 3 i + d of the element, i < 20; rows 60 + d hold the
// direction sums of the stored rows (sum over i of row 3 i + d, for the mean
// translation of the result); row 63 and columns 60..63 are zero.  The tile
// is stored as it sits in shared memory, followed by 1 / s_e (FP32) and 12
// zero bytes: 16,400 bytes per element, one bulk copy.
constexpr int kTileA = 8192;                  // one term of the A tile (64 rows)
constexpr int kRecBytes = 2 * kTileA + 16;    // 16400
constexpr int kRecStage = 2 * kTileA + 128;   // bytes of one record stage (16,512)

// dof of the element for direction-ordered row or column r < 60
__host__ __device__ constexpr int dir_dof(int r) { return 3 * (r % 20) + r / 20; }

// ---- pipeline of the tensor-core kernel ------------------------------------
constexpr int kNAcc = 4;             // TMEM accumulators (128 columns each)
constexpr int kAccCols = 128;
constexpr int kEpiGroups = 2;        // warps 0-7: two epilogue groups of four warps on alternate elements;
constexpr int kEpiWarps = 4;         //   warp w reads TMEM lanes 32 (w % 4) .. +31 = rows 32 (w % 4) .. +31
constexpr int kBldWarp0 = 8;         // warps 8 .. 8 + np - 1 build the B tiles, warp 8 + w the elements
constexpr int kBldWarps = 8;         //   t = w (mod np), from P stage w into tile set w (np <= 8)
constexpr int kProdWarp = 16;        // warp 16 copies the element records, warps 17-18 gather P
constexpr int kGatherWarps = 2;      //   on alternate elements (np even: one warp fills each P stage)
constexpr int kMaxRec = 12;          // record stages
constexpr int kMmaWarp = 19;         // warp 19, lane 0 issues the MMAs
constexpr int kH16Threads = 20 * 32;
static_assert(kBldWarp0 + kBldWarps == kProdWarp, "warp roles overlap");

// shared-memory plan for kb cases per pass and nr record stages
struct Plan {
    int kb, nr;
    int np;        // P stages = tile sets = builder warps
    int pst;       // bytes of one P stage: P of the 20 nodes, then 1/s_e (16 B)
    int tile;      // bytes of one tile set: B (2 terms), the per-case output scales
    int off_p, off_tile, off_aux, smem;
};

// P stages per pass width: the builders' B tiles cost more than a deeper
// record ring buys (measured at 8 to 64 cases on GB300)
__host__ __device__ constexpr int plan_np(int kb) { return kb <= 16 ? 8 : kb == 32 ? 6 : 4; }
static_assert(plan_np(8) % kGatherWarps == 0 && plan_np(16) % kGatherWarps == 0 &&
                  plan_np(32) % kGatherWarps == 0 && plan_np(64) % kGatherWarps == 0,
              "each P stage must have one gather warp");

__host__ __device__ inline Plan make_plan(int kb, int nr)
{
    Plan p;
    p.kb = kb;
    p.nr = nr;
    p.np = plan_np(kb);
    p.pst = 480 * kb + 128;
    p.tile = 256 * kb + 256;
    p.off_p = nr * kRecStage;
    p.off_tile = p.off_p + p.np * p.pst;
    p.off_aux = p.off_tile + p.np * p.tile;
    // aux: mbarriers (64 words), tmem slot, flags and counters (128 B), per
    // epilogue group two sets of sum rows (2 x 3 x 64 floats)
    p.smem = p.off_aux + 64 * 8 + 128 + kEpiGroups * 6 * kMaxKB * 4;
    // at least half the SM's shared memory, so that one CTA holds an SM (its
    // TMEM allocation takes all 512 columns)
    if (p.smem < 116 * 1024) p.smem = 116 * 1024;
    return p;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void named_sync(int id, int n)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// (a, b) = hi + lo in FP16, both rounded to nearest even: the words of the
// two terms, (a_hi, b_hi) and (a_lo, b_lo), a in the low half-word.
__device__ __forceinline__ void split2_f16(float a, float b, uint32_t &w_hi, uint32_t &w_lo)
{
    const __half ha = __float2half_rn(a), hb = __float2half_rn(b);
    const float ra = a - __half2float(ha), rb = b - __half2float(hb);
    w_hi = (uint32_t)__half_as_ushort(ha) | ((uint32_t)__half_as_ushort(hb) << 16);
    w_lo = cvt_f16x2(ra, rb);
}

}  // namespace

// ---------------------------------------------------------------------------
// Set-up: the element records of the tensor-core product from FP64 storkm.
// One 128-thread block per element (grid-stride): s_e = 2^(14 - E) with
// max |K_e| (and max |direction sum|) < 2^E, the two FP16 terms of every
// scaled entry, the direction sums of the stored (rounded) rows formed in
// FP64 from hi + lo and split in turn, then the two terms' tiles.
__global__ void __launch_bounds__(128) k_mr_pack(int nels, const double *__restrict__ km, unsigned char *__restrict__ rec)
{
    __shared__ uint32_t t2[64 * 64];   // (hi, lo) half pairs of the 64 x 64 tile, row-major
    __shared__ double red[4];
    const int tid = threadIdx.x;
    for (int e = blockIdx.x; e < nels; e += gridDim.x) {
        const double *ke = km + (size_t)e * 3600;
        double mx = 0.0;
        for (int q = tid; q < 3600; q += 128) mx = fmax(mx, fabs(ke[q]));
        for (int q = tid; q < 3 * 60; q += 128) {   // the direction sums must fit FP16 too
            const int d = q / 60, c = q % 60;
            double sum = 0.0;
            for (int i = 0; i < 20; ++i) sum += ke[60 * c + 3 * i + d];
            mx = fmax(mx, fabs(sum));
        }
        mx = warp_max(mx);
        if ((tid & 31) == 0) red[tid >> 5] = mx;
        __syncthreads();
        mx = fmax(fmax(red[0], red[1]), fmax(red[2], red[3]));
        int ex = 0;
        frexp(mx, &ex);                              // mx < 2^ex
        const double sc = mx > 0.0 ? ldexp(1.0, 14 - ex) : 1.0;
        for (int q = tid; q < 64 * 64; q += 128) {
            const int r = q / 64, c = q % 64;
            float x = 0.f;
            if (r < 60 && c < 60) x = (float)(ke[60 * c + dir_dof(r)] * sc);
            uint32_t wh, wl;
            split2_f16(x, 0.f, wh, wl);
            t2[q] = (wh & 0xffffu) | (wl << 16);
        }
        __syncthreads();
        // rows 60..62: sums over i of the stored rows 20 d + i
        for (int q = tid; q < 3 * 60; q += 128) {
            const int d = q / 60, c = q % 60;
            double s = 0.0;
            for (int i = 0; i < 20; ++i) {
                const uint32_t w = t2[(20 * d + i) * 64 + c];
                s += (double)__half2float(__ushort_as_half((unsigned short)(w & 0xffffu))) +
                     (double)__half2float(__ushort_as_half((unsigned short)(w >> 16)));
            }
            uint32_t wh, wl;
            split2_f16((float)s, 0.f, wh, wl);
            t2[(60 + d) * 64 + c] = (wh & 0xffffu) | (wl << 16);
        }
        __syncthreads();
        // the A tile: 2 terms x 8 x 8 core matrices x 8 rows of 16 bytes
        unsigned char *out = rec + (size_t)e * kRecBytes;
        for (int q = tid; q < 2 * 64 * 8; q += 128) {
            const int term = q / 512, rem = q % 512, I = rem / 64, J = (rem / 8) % 8, rr = rem % 8;
            const int row = 8 * I + rr;
            uint32_t w[4];
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const uint32_t a = t2[row * 64 + 8 * J + 2 * g], b = t2[row * 64 + 8 * J + 2 * g + 1];
                w[g] = term == 0 ? ((a & 0xffffu) | (b << 16)) : ((a >> 16) | (b & 0xffff0000u));
            }
            *reinterpret_cast<uint4 *>(out + term * kTileA + I * 1024 + J * 128 + rr * 16) =
                make_uint4(w[0], w[1], w[2], w[3]);
        }
        if (tid == 0) {
            float *tail = reinterpret_cast<float *>(out + 2 * kTileA);
            tail[0] = (float)(1.0 / sc);
            tail[1] = tail[2] = tail[3] = 0.f;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Block element products on the tensor cores, cases c0 .. c0+KB-1 of k:
// ut[e][i][c0 + j] = (P K_e (P_e - t_j))(i, j), t_j a translation of case j
// and P removing each case's mean translation from the result over the
// element's 20 nodes (identities in exact arithmetic, since K_e annihilates
// rigid translations; with rounded operands they keep the rounding away
// from the smooth part of P and the product symmetric, as the single-case
// kernels do).
//
// One persistent CTA of 20 warps per SM walks the elements e = blockIdx.x +
// t * gridDim.x with warp-specialised roles linked by mbarriers.  The
// element records, the stream that HBM bounds, have a ring of their own
// (nr stages) that only the copy warp and the MMA hold, so that most of it
// is in flight at any time; P and the B tiles have a second ring (np
// stages, one per builder warp):
//   warp 16     one thread copies the element record (the A tile of both
//               terms and 1/s_e) by one bulk copy (cp.async.bulk) into the
//               record ring;
//   warps 17-18 on alternate elements gather the P rows of the element's 20
//               nodes (FP32 high and low parts, kept beside P by the update
//               kernels) by TMA gathers of four rows each (one row per node
//               when a pass covers all k cases, else one per node and
//               direction), and 1/s_e from the record's tail, into the P
//               ring;
//   warps 8-15  warp 8 + w (w < np) builds the B tiles of the elements
//               t = w (mod np) from P stage w into tile set w: per case j a
//               translation t_j (node 0's value) and a power-of-two scale s_j
//               (the case's largest |p - t_j| met in warp shuffles), then
//               (P_e - t_j) s_j split into two FP16 terms, the high term's KB
//               rows followed by the low term's;
//   warp 19     one thread issues [A_hi; A_lo] x [B_hi | B_lo] (M = 128,
//               N = 2 KB, four K-steps, A from the record stage, B from the
//               tile) into a ring of kNAcc TMEM accumulators and commits them
//               to mbarriers that free the record stage and fill the
//               accumulator;
//   warps 0-7   two groups of four warps on alternate elements read the
//               accumulator back (warp w: TMEM lanes 32 (w % 4) .. +31, which
//               hold row 32 (w % 4) + lane of D), add each row's two column
//               halves, pass the low-term rows 64..127 through the tile's B
//               region (the MMA is done with it) to the high-term rows,
//               subtract a twentieth of the direction's sum row, undo the
//               scales, store, and free the tile.
// Each ring is filled by one warp in element order and every barrier is
// waited on by one thread that passes its phases in turn, so no parity wait
// can run two phases ahead.
// Every wait is bounded; where a group of warps meets at a named barrier,
// one thread waits and the group follows its outcome.  A wait that runs out
// sets a shared failure flag that every role checks before its next wait,
// writes 3 to the device error word, and the CTA waits (bounded) for the
// copies and MMAs it has in flight before it frees its TMEM and returns.
//
// tmap: P as 2-D FP64-sized elements, rows of one node (3 KB elements, box
// 3 KB x 1) when whole != 0, else rows of one slot (k elements, box KB x 1,
// gathered from column c0).
template <int KB>
__global__ void __launch_bounds__(kH16Threads, 1)
k_mr_elem_h16(int nels, int k, int c0, int nr, const unsigned char *__restrict__ rec,
              const int *__restrict__ conn, const __grid_constant__ CUtensorMap tmap, int whole,
              float *__restrict__ ut, int *__restrict__ err, const int *__restrict__ skip)
{
    constexpr int kb = KB;
    if (skip && *skip) return;   // a residual replacement is pending: nothing to compute
    extern __shared__ __align__(1024) unsigned char sm[];
    const Plan pl = make_plan(kb, nr);
    const int np = pl.np;
    unsigned char *rstg = sm;                  // record stages
    unsigned char *pstg = sm + pl.off_p;       // P stages
    unsigned char *tiles = sm + pl.off_tile;   // B tile sets
    uint64_t *rc_full = reinterpret_cast<uint64_t *>(sm + pl.off_aux);
    uint64_t *rc_empty = rc_full + kMaxRec;
    uint64_t *pp_full = rc_empty + kMaxRec;
    uint64_t *pp_empty = pp_full + 8;
    uint64_t *tl_full = pp_empty + 8;
    uint64_t *tl_empty = tl_full + 8;
    uint64_t *ac_full = tl_empty + 8;
    uint64_t *ac_empty = ac_full + kNAcc;      // 64 words in all
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + pl.off_aux + 64 * 8);
    volatile int *s_fail = reinterpret_cast<volatile int *>(tslot + 1);
    int *s_count = reinterpret_cast<int *>(tslot + 2);          // [1] MMA groups committed
    volatile int *g_ok = reinterpret_cast<volatile int *>(tslot + 4);     // [epi group][element parity]: waits passed
    volatile int *r_last = reinterpret_cast<volatile int *>(tslot + 8);   // [record stage]: last element copied in
    volatile int *p_last = reinterpret_cast<volatile int *>(tslot + 20);  // [P stage]: last element gathered in
    float *e_aux = reinterpret_cast<float *>(sm + pl.off_aux + 64 * 8 + 128);   // [epi group][parity][d][j]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nmine = blockIdx.x < nels ? (nels - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto elem = [&](int t) { return (int)blockIdx.x + t * (int)gridDim.x; };

    if (warp == 0) tmem_alloc(tslot, kNAcc * kAccCols);
    if (tid == 0) {
        for (int i = 0; i < nr; ++i) {
            mbar_init(&rc_full[i], 1);            // the record warp's arrival (with the bytes it expects)
            mbar_init(&rc_empty[i], 1);           // the MMA's commit (A read)
        }
        for (int i = 0; i < np; ++i) {
            mbar_init(&pp_full[i], 1);            // the gather warp's arrival (with the bytes it expects)
            mbar_init(&pp_empty[i], 1);           // the builder warp, done reading P
            mbar_init(&tl_full[i], 1);            // the builder warp, done writing B
            mbar_init(&tl_empty[i], kEpiWarps);   // the four epilogue warps that used the tile last
        }
        for (int i = 0; i < kNAcc; ++i) {
            mbar_init(&ac_full[i], 1);
            mbar_init(&ac_empty[i], kEpiWarps);
        }
        mbar_fence_init();
        *s_fail = 0;
        s_count[0] = s_count[1] = 0;
        for (int i = 0; i < 4; ++i) g_ok[i] = 0;
        for (int i = 0; i < kMaxRec; ++i) r_last[i] = -1;
        for (int i = 0; i < 8; ++i) p_last[i] = -1;
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    auto wait = [&](uint64_t *bar, uint32_t parity) {
        if (*s_fail) return false;
        if (mbar_wait(bar, parity)) return true;
        *s_fail = 1;
        return false;
    };

    if (warp == kProdWarp) {
        // the element records (A tile, 1/s_e), one bulk copy each, into the
        // ring of nr record stages
        if (lane == 0) {
            int r = 0, lap = 0;   // t = lap * nr + r (nr is a launch parameter: no division per element)
            for (int t = 0; t < nmine; ++t) {
                if (t >= nr && !wait(&rc_empty[r], (uint32_t)((lap - 1) & 1))) break;
                mbar_expect_tx(&rc_full[r], kRecBytes);
                bulk_g2s(rstg + (size_t)r * kRecStage, rec + (size_t)elem(t) * kRecBytes, kRecBytes, &rc_full[r]);
                r_last[r] = t;   // for the drain after a failure
                if (++r == nr) {
                    r = 0;
                    ++lap;
                }
            }
        }
        __syncwarp();
    } else if (warp > kProdWarp && warp <= kProdWarp + kGatherWarps) {
        // gather warp gw takes the elements t = gw (mod 2): the P rows of the
        // element's 20 nodes (FP32 high and low parts) by TMA gathers of four
        // rows, and 1/s_e from the record's tail, into P stage t % np.  Whole:
        // lane g < 5 takes nodes 4g..4g+3; else lane g < 15 takes the
        // node-direction rows r = 4g..4g+3 (node r / 3, direction r % 3).  Each
        // lane loads its own rows' nodes, kCD elements ahead.
        const int gw = warp - kProdWarp - 1;
        const int ngat = whole ? 5 : 15;
        const int rowbytes = whole ? 24 * kb : 8 * kb;
        const uint32_t pbytes = 480 * kb;
        auto rows_of = [&](int t) {
            int4 v = make_int4(0, 0, 0, 0);
            if (t < nmine && lane < ngat) {
                const int *ce = conn + (size_t)elem(t) * 20;
                if (whole) {
                    v = *reinterpret_cast<const int4 *>(ce + 4 * lane);
                } else {
                    const int r = 4 * lane;
                    v = make_int4(3 * ce[r / 3] + r % 3, 3 * ce[(r + 1) / 3] + (r + 1) % 3,
                                  3 * ce[(r + 2) / 3] + (r + 2) % 3, 3 * ce[(r + 3) / 3] + (r + 3) % 3);
                }
            }
            return v;
        };
        constexpr int kCD = 4;
        int4 nd[kCD];
#pragma unroll
        for (int j = 0; j < kCD; ++j) nd[j] = rows_of(gw + kGatherWarps * j);
        bool stop = false;
        for (int t0 = gw; t0 < nmine && !stop; t0 += kGatherWarps * kCD) {
#pragma unroll
            for (int j = 0; j < kCD; ++j) {
                const int t = t0 + kGatherWarps * j;
                if (t >= nmine) break;
                const int w = t % np;
                int ok = 1;
                if (t >= np && lane == 0 && !mbar_test(&pp_empty[w], (uint32_t)((t / np - 1) & 1)))
                    ok = wait(&pp_empty[w], (uint32_t)((t / np - 1) & 1)) ? 1 : 0;
                if (!__shfl_sync(kFullMask, ok, 0)) {
                    stop = true;
                    break;
                }
                if (lane == 0) mbar_expect_tx(&pp_full[w], pbytes + 16);
                __syncwarp();
                unsigned char *dst = pstg + (size_t)w * pl.pst;
                if (lane < ngat)
                    tma_gather4(dst + lane * 4 * rowbytes, &tmap, whole ? 0 : c0, nd[j].x, nd[j].y, nd[j].z, nd[j].w,
                                &pp_full[w]);
                if (lane == 31) bulk_g2s(dst + pbytes, rec + (size_t)elem(t) * kRecBytes + 2 * kTileA, 16, &pp_full[w]);
                nd[j] = rows_of(t + kGatherWarps * kCD);
                if (lane == 0) p_last[w] = t;   // for the drain after a failure
            }
        }
    } else if (warp >= kBldWarp0 && warp < kBldWarp0 + np) {
        // Warp w builds the B tiles of the elements t = w (mod np), so that
        // it alone waits on P stage w and tile set w and passes each of their
        // mbarrier phases in turn (a parity wait must never run two phases
        // ahead).  Lane l takes case j = l % kb (kb <= 32;
        // case 32 c + l of slice c for kb = 64) and the K-column chunks of
        // eight q = l / kb + L m, so that the lanes of one case meet in
        // shuffles for the case's largest |p - t_j|.  The K columns are the
        // element's dofs in their natural order (c = 3 i + d), so column c of
        // B row j is P row c of the stage: every load is a fixed offset from
        // the lane's base.
        constexpr int L = kb >= 32 ? 1 : 32 / kb;   // lanes per case
        constexpr int NQ = 8 / L;                   // chunks per lane
        constexpr int NS = kb > 32 ? kb / 32 : 1;   // case slices
        constexpr bool kRegs = NQ <= 4;             // up to 16 cases: the values stay in registers
        const int w = warp - kBldWarp0;
        const int q0 = NS > 1 ? 0 : lane / kb;
        const bool tail = q0 == L - 1;              // this lane's last chunk holds columns 56..63 (60..63 zero)
        const int dbase = (2 * q0) % 3;             // direction of column 8 q0
        for (int t = w; t < nmine; t += np) {
            const uint32_t ph = (uint32_t)((t / np) & 1);
            int ok = 1;
            if (lane == 0 && !(mbar_test(&pp_full[w], ph) & (t < np || mbar_test(&tl_empty[w], ph ^ 1u))))
                ok = wait(&pp_full[w], ph) && (t < np || wait(&tl_empty[w], ph ^ 1u));
            if (!__shfl_sync(kFullMask, ok, 0)) break;
            const unsigned char *S = pstg + (size_t)w * pl.pst;
            const float2 *Pe = reinterpret_cast<const float2 *>(S);   // [dof][j]: hi, lo
            const float inv_se = *reinterpret_cast<const float *>(S + 480 * kb);
            unsigned char *B = tiles + (size_t)w * pl.tile;
            float *oscale = reinterpret_cast<float *>(B + 256 * kb);   // per case: 1 / (s_e s_j)
#pragma unroll
            for (int cs = 0; cs < NS; ++cs) {
                const int j = NS > 1 ? 32 * cs + lane : lane % kb;
                // the translation t_j: node 0's value (any translation serves);
                // u[r] is the one of column 8 q0 + r (mod 3)
                float t3[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) t3[d] = Pe[d * kb + j].x;
                const float u[3] = {dbase == 0 ? t3[0] : dbase == 1 ? t3[1] : t3[2],
                                    dbase == 0 ? t3[1] : dbase == 1 ? t3[2] : t3[0],
                                    dbase == 0 ? t3[2] : dbase == 1 ? t3[0] : t3[1]};
                const float2 *Pj = Pe + (size_t)(8 * q0) * kb + j;
                // p - t_j at column 8 (q0 + L m) + g (zero past 60)
                auto val = [&](int m, int g) {
                    if (m == NQ - 1 && g >= 4 && tail) return 0.f;
                    const float2 v = Pj[(8 * L * m + g) * kb];
                    return (v.x - u[(8 * L * m + g) % 3]) + v.y;
                };
                float xv[kRegs ? NQ : 1][8];
                float mx = 0.f;
#pragma unroll
                for (int m = 0; m < NQ; ++m)
#pragma unroll
                    for (int g = 0; g < 8; ++g) {
                        const float x = val(m, g);
                        if constexpr (kRegs) xv[m][g] = x;
                        mx = fmaxf(mx, fabsf(x));
                    }
#pragma unroll
                for (int o = kb; o < 32; o <<= 1) mx = fmaxf(mx, __shfl_xor_sync(kFullMask, mx, o));
                // s_j = 2^(14 - E) with max |p - t_j| < 2^E
                int ex = 0;
                frexpf(mx, &ex);
                const float sj = mx > 0.f ? ldexpf(1.f, 14 - ex) : 1.f;
                if (q0 == 0) oscale[j] = inv_se / sj;
                // B tile: row j (case), K-columns 8 q .. 8 q + 7; the low
                // term's rows follow the high term's (rows kb + j)
#pragma unroll
                for (int m = 0; m < NQ; ++m) {
                    const int q = q0 + L * m;
                    float x8[8];
#pragma unroll
                    for (int g = 0; g < 8; ++g) x8[g] = (kRegs ? xv[kRegs ? m : 0][g] : val(m, g)) * sj;
                    uint32_t wh[4], wl[4];
#pragma unroll
                    for (int g = 0; g < 4; ++g) split2_f16(x8[2 * g], x8[2 * g + 1], wh[g], wl[g]);
                    const uint32_t off = kmajor_off(j, 8 * q);
                    *reinterpret_cast<uint4 *>(B + off) = make_uint4(wh[0], wh[1], wh[2], wh[3]);
                    *reinterpret_cast<uint4 *>(B + 128 * kb + off) = make_uint4(wl[0], wl[1], wl[2], wl[3]);
                }
            }
            fence_proxy_async();   // this lane's tile writes -> the tensor cores
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&pp_empty[w]);   // P read: the stage may be refilled
                mbar_arrive(&tl_full[w]);
            }
        }
    } else if (warp == kMmaWarp) {
        int t = 0;
        if (lane == 0) {
            // kind::f16 with both operands FP16 (the format is in the instruction descriptor)
            const uint32_t idesc = idesc_f16(128, 2u * kb);
            int r = 0, rlap = 0;   // t = rlap * nr + r (no division per element)
            for (; t < nmine; ++t) {
                const int b = t % np, a = t % kNAcc;
                const uint32_t pr = (uint32_t)(rlap & 1), pb = (uint32_t)((t / np) & 1),
                               pa = (uint32_t)((t / kNAcc - 1) & 1);
                // the three barriers tested at once; the bounded waits only when one is not ready
                const bool ready = mbar_test(&rc_full[r], pr) & mbar_test(&tl_full[b], pb) &
                                   (t < kNAcc || mbar_test(&ac_empty[a], pa));
                if (!ready) {
                    if (!wait(&rc_full[r], pr)) break;
                    if (!wait(&tl_full[b], pb)) break;
                    if (t >= kNAcc && !wait(&ac_empty[a], pa)) break;
                }
                tc_fence_after();
                const uint32_t a0 = smem_u32(rstg + (size_t)r * kRecStage);
                const uint32_t b0 = smem_u32(tiles + (size_t)b * pl.tile);
                const uint32_t d0 = tmem + (uint32_t)(kAccCols * a);
                // [A_hi; A_lo] x [B_hi | B_lo]: the four products of the two splits
#pragma unroll
                for (int ks = 0; ks < 4; ++ks)   // K = 64 in steps of 16 (two core matrices)
                    mma_bf16(d0, umma_desc(a0 + ks * 256, 128, 1024), umma_desc(b0 + ks * 256, 128, 1024), idesc,
                             ks > 0 ? 1u : 0u);
                mma_commit(&rc_empty[r]);
                mma_commit(&ac_full[a]);
                if (++r == nr) {
                    r = 0;
                    ++rlap;
                }
            }
            s_count[1] = t;
        }
        __syncwarp();
    } else if (warp < kEpiGroups * kEpiWarps) {
        // group eg takes the elements t = eg, eg + 2, ...; lane l of its warp
        // q = warp % 4 holds row 32q + l of D: rows 0..63 are the high term's
        // products of the direction-ordered rows, rows 64..127 the low term's
        const int eg = warp / kEpiWarps, q = warp % kEpiWarps, et = tid - eg * kEpiWarps * 32;
        const int row = 32 * (q & 1) + lane;        // the element row this lane adds into
        const int dn = row < 60 ? row / 20 : 0;
        const int bar_id = 6 + eg;
        for (int t = eg; t < nmine; t += kEpiGroups) {
            const int a = t % kNAcc, b = t % np, kk = t / kEpiGroups;
            if (et == 0) g_ok[2 * eg + (kk & 1)] = wait(&ac_full[a], (uint32_t)((t / kNAcc) & 1));
            named_sync(bar_id, kEpiWarps * 32);
            if (!g_ok[2 * eg + (kk & 1)]) break;
            tc_fence_after();
            // 32 columns per load, each load with its wait in one asm statement
            // (the registers are defined only once the wait has returned); the
            // accumulator's columns j and kb + j add up to case j
            const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(kAccCols * a);
            float v[kb];
            if constexpr (kb <= 16) {
                float w[32];
                tmem_ld_32x32b_x32(ta, w);
#pragma unroll
                for (int j = 0; j < kb; ++j) v[j] = w[j] + w[kb + j];
            } else {
#pragma unroll
                for (int c = 0; c < kb / 32; ++c) {
                    float w[32];
                    tmem_ld_32x32b_x32(ta + 32 * c, w);
#pragma unroll
                    for (int i = 0; i < 32; ++i) v[32 * c + i] = w[i];
                }
#pragma unroll
                for (int c = 0; c < kb / 32; ++c) {
                    float w[32];
                    tmem_ld_32x32b_x32(ta + kb + 32 * c, w);
#pragma unroll
                    for (int i = 0; i < 32; ++i) v[32 * c + i] += w[i];
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ac_empty[a]);
            // the low-term rows pass through the tile's B region (64 rows x kb floats)
            unsigned char *T = tiles + (size_t)b * pl.tile;
            float *xl = reinterpret_cast<float *>(T);
            if (q >= 2) {
#pragma unroll
                for (int j = 0; j < kb; ++j) xl[row * kb + j] = v[j];
            }
            named_sync(bar_id, kEpiWarps * 32);
            float *es = e_aux + (eg * 2 + (kk & 1)) * 3 * kMaxKB;
            if (q < 2) {
#pragma unroll
                for (int j = 0; j < kb; ++j) v[j] += xl[row * kb + j];
                // the sum rows 60..62: lanes 28..30 of warp 1
                if (q == 1 && lane >= 28 && lane < 31) {
#pragma unroll
                    for (int j = 0; j < kb; ++j) es[(lane - 28) * kMaxKB + j] = v[j];
                }
            }
            named_sync(bar_id, kEpiWarps * 32);
            const float *osc = reinterpret_cast<const float *>(T + 256 * kb);
            if (q < 2 && row < 60) {
                float *o = ut + ((size_t)elem(t) * 60 + dir_dof(row)) * k + c0;
#pragma unroll
                for (int j4 = 0; j4 < kb; j4 += 4) {
                    float4 w;
                    w.x = (v[j4] - 0.05f * es[dn * kMaxKB + j4]) * osc[j4];
                    w.y = (v[j4 + 1] - 0.05f * es[dn * kMaxKB + j4 + 1]) * osc[j4 + 1];
                    w.z = (v[j4 + 2] - 0.05f * es[dn * kMaxKB + j4 + 2]) * osc[j4 + 2];
                    w.w = (v[j4 + 3] - 0.05f * es[dn * kMaxKB + j4 + 3]) * osc[j4 + 3];
                    *reinterpret_cast<float4 *>(o + j4) = w;
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&tl_empty[b]);   // the tile is free for the next B operand
        }
    }
    __syncthreads();
    if (*s_fail) {
        if (tid == 0) {
            atomicExch(err, 3);
            // Wait (bounded) for the copies and MMAs still in flight: the last
            // copy into each stage (a stage is refilled only after its
            // previous copy was consumed) and the last MMA commit (it
            // completes after every MMA issued before it).
            for (int i = 0; i < nr; ++i) {
                const int t = r_last[i];
                if (t >= 0) mbar_wait(&rc_full[i], (uint32_t)((t / nr) & 1));
            }
            for (int i = 0; i < np; ++i) {
                const int t = p_last[i];
                if (t >= 0) mbar_wait(&pp_full[i], (uint32_t)((t / np) & 1));
            }
            const int tm = s_count[1] - 1;
            if (tm >= 0) mbar_wait(&ac_full[tm % kNAcc], (uint32_t)((tm / kNAcc) & 1));
        }
        __syncthreads();
    }
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, kNAcc * kAccCols);
}

// Block element products on CUDA cores (FP32 or FP64): one warp per element,
// lanes own rows 2l, 2l+1; the cases in chunks of 8, each chunk's P_e staged
// in shared memory per warp.
template <typename KT, typename OT>
__global__ void __launch_bounds__(256)
k_mr_elem_cc(int nels, int k, const KT *__restrict__ km, const int *__restrict__ conn, const double *__restrict__ P,
             OT *__restrict__ ut, const int *__restrict__ skip)
{
    constexpr int CB = 8;
    __shared__ KT ps[8][60 * CB];
    if (skip && *skip) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int e = warp; e < nels; e += nwarps) {
        for (int cc = 0; cc < k; cc += CB) {
            for (int idx = lane; idx < 60 * CB; idx += 32) {
                const int c = idx / CB, j = idx - CB * c;
                const int nd = conn[(size_t)e * 20 + c / 3];
                ps[w][idx] = (KT)P[((size_t)3 * nd + c % 3) * k + cc + j];
            }
            __syncwarp();
            if (lane < 30) {
                KT a0[CB], a1[CB];
#pragma unroll
                for (int j = 0; j < CB; ++j) a0[j] = a1[j] = (KT)0;
                const KT *ke = km + (size_t)e * 3600 + 2 * lane;
                for (int c = 0; c < 60; ++c) {
                    const KT k0 = ke[60 * c], k1 = ke[60 * c + 1];
#pragma unroll
                    for (int j = 0; j < CB; ++j) {
                        const KT pj = ps[w][c * CB + j];
                        a0[j] = fma(k0, pj, a0[j]);
                        a1[j] = fma(k1, pj, a1[j]);
                    }
                }
                OT *o0 = ut + ((size_t)e * 60 + 2 * lane) * k + cc;
#pragma unroll
                for (int j = 0; j < CB; ++j) {
                    o0[j] = (OT)a0[j];
                    o0[k + j] = (OT)a1[j];
                }
            }
            __syncwarp();
        }
    }
}

// Threads of the block kernels over (slot or node, case): a multiple of k,
// so that a thread's case j = threadIdx.x % k stays fixed in the
// grid-stride loop.
__host__ __device__ inline int case_threads(int k) { return k * (256 / k); }

// Sums NV per-thread values over the threads of each case in thread order
// (kinds bit = max) and writes part[v * stride + blockIdx.x * k + j].
template <int NV>
__device__ __forceinline__ void case_block_reduce(double (&v)[NV], unsigned kinds, double *out, size_t stride, int k)
{
    __shared__ double sh[NV][256];
#pragma unroll
    for (int q = 0; q < NV; ++q) sh[q][threadIdx.x] = v[q];
    __syncthreads();
    if ((int)threadIdx.x < k) {
        const int ng = blockDim.x / k;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = 0.0;
            for (int g = 0; g < ng; ++g) {
                const double x = sh[q][g * k + threadIdx.x];
                s = ((kinds >> q) & 1) ? fmax(s, x) : s + x;
            }
            out[q * stride + (size_t)blockIdx.x * k + threadIdx.x] = s;
        }
    }
    __syncthreads();
}

// Node scatter for k load cases: thread (node, j), ascending element order.
// MODE 0: U = sum, partial p.u per case; MODE 1: RRES = F - sum, partial rr.
template <typename UT, int MODE>
__global__ void __launch_bounds__(256)
k_mr_scatter(int nn, int k, const int *__restrict__ ptr, const int *__restrict__ list, const UT *__restrict__ ut,
             const uint8_t *__restrict__ fm, const double *__restrict__ pf, double *__restrict__ out,
             double *__restrict__ part, const int *__restrict__ skip)
{
    if (skip && *skip) return;   // uniform: the flag does not change during the kernel
    const int j = threadIdx.x % k;
    double loc = 0.0;
    // the block size is a multiple of k: a thread's case stays j and its
    // node advances by the stride over k (no division in the loop)
    const size_t stride = (size_t)gridDim.x * blockDim.x, t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int dn = (int)(stride / k);
    int n = (int)(t0 / k);
    for (size_t t = t0; t < (size_t)nn * k; t += stride, n += dn) {
        UT a0 = 0, a1 = 0, a2 = 0;   // FP32 products are summed in FP32, FP64 ones in FP64
        for (int q = ptr[n]; q < ptr[n + 1]; ++q) {
            const size_t base = (size_t)list[q] * 3 * k + j;   // list holds e*20+a
            a0 += ut[base];
            a1 += ut[base + k];
            a2 += ut[base + 2 * k];
        }
        const int m = fm[n];
        const double a[3] = {(double)a0, (double)a1, (double)a2};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const size_t s = ((size_t)3 * n + d) * k + j;
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
    double v[1] = {loc};
    case_block_reduce<1>(v, 0u, part, 0, k);
}

// per-case state
struct MState {
    double up[kMaxK], ff[kMaxK], rr[kMaxK], thr[kMaxK];
    double alpha[kMaxK], beta[kMaxK];   // this iteration's step lengths (0 for inactive cases)
    int active[kMaxK];   // 1 until the case's true residual reaches tol
    int flag[kMaxK];     // recursive residual reached thr (replacement wanted)
    int iters[kMaxK];
    int any_flag;        // stop iterating: some active case wants a replacement
    int pending;         // set by this iteration's k_mr_beta, moved to any_flag by k_mr_finish
    int err;
};

// per-case sums of block partials (fixed order)
__device__ __forceinline__ double case_sum(const double *part, int G, int j, int k)
{
    double s = 0.0;
    for (int b = 0; b < G; ++b) s += part[(size_t)b * k + j];
    return s;
}

// The same sums by one 256-thread block: thread (g, j) adds partials g, g+ng,
// ... of case j (ng = 256 / k groups), then thread j adds the ng group sums
// in order.  Fixed order, so the result is the same in every run.  Valid in
// threads 0..k-1.
__device__ __forceinline__ double case_sum_block(const double *part, int G, double *sh, int k)
{
    const int ng = 256 / k;
    const int j = threadIdx.x % k, g = threadIdx.x / k;
    double s = 0.0;
    if (g < ng)
        for (int b = g; b < G; b += ng) s += part[(size_t)b * k + j];
    sh[threadIdx.x] = s;
    __syncthreads();
    double t = 0.0;
    if ((int)threadIdx.x < k)
        for (int i = 0; i < ng; ++i) t += sh[i * k + threadIdx.x];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(256)
k_mr_init(int ns, int k, const double *__restrict__ F, const double *__restrict__ dinv, double *__restrict__ X,
          double *__restrict__ R, double *__restrict__ D, double *__restrict__ P, float2 *__restrict__ Ps,
          double *__restrict__ part, int G)
{
    double rd = 0.0, rr = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x, t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t ds = stride / k;   // the block size is a multiple of k
    size_t s = t0 / k;
    for (size_t t = t0; t < (size_t)ns * k; t += stride, s += ds) {
        const double rv = F[t], dv = dinv[s] * rv;
        X[t] = 0.0;
        R[t] = rv;
        D[t] = dv;
        P[t] = dv;
        float h, l;
        split_f64(dv, h, l);
        Ps[t] = make_float2(h, l);
        rd = fma(rv, dv, rd);
        rr = fma(rv, rv, rr);
    }
    double v[2] = {rd, rr};
    case_block_reduce<2>(v, 0u, part, (size_t)G * k, k);
}

__global__ void k_mr_init2(MState *st, const double *__restrict__ part, int G, int k, double tol)
{
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        const double rd = case_sum(part, G, j, k), rr = case_sum(part + (size_t)G * k, G, j, k);
        st->up[j] = rd;
        st->ff[j] = rr;
        st->rr[j] = rr;
        st->thr[j] = 0.1 > tol ? 0.1 : tol;
        st->active[j] = rr > 0.0 ? 1 : 0;
        st->flag[j] = 0;
        st->iters[j] = 0;
    }
    if (threadIdx.x == 0) {
        st->any_flag = 0;
        st->pending = 0;
        st->err = 0;
    }
}

// alpha = up / (p.u) per case, from the scatter's partials (one block)
__global__ void __launch_bounds__(256) k_mr_alpha(MState *st, const double *__restrict__ ps, int Gs, int k)
{
    __shared__ double sh[256];
    if (st->any_flag) return;
    const double pu = case_sum_block(ps, Gs, sh, k);
    const int j = threadIdx.x;
    if (j < k) st->alpha[j] = st->active[j] ? st->up[j] / pu : 0.0;
}

__global__ void __launch_bounds__(256)
k_mr_update1(int ns, int k, const MState *__restrict__ st, double *__restrict__ pu_out, int G, double *__restrict__ X,
             double *__restrict__ R, double *__restrict__ D, const double *__restrict__ P,
             const double *__restrict__ U, const double *__restrict__ dinv)
{
    if (st->any_flag) return;
    const int j = threadIdx.x % k;
    const double alpha = st->alpha[j];
    double rd = 0.0, rr = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x, t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t ds = stride / k;   // the block size is a multiple of k
    size_t s = t0 / k;
    for (size_t t = t0; t < (size_t)ns * k; t += stride, s += ds) {
        X[t] = fma(P[t], alpha, X[t]);
        const double rn = fma(-U[t], alpha, R[t]);
        R[t] = rn;
        const double dn = dinv[s] * rn;
        D[t] = dn;
        rd = fma(rn, dn, rd);
        rr = fma(rn, rn, rr);
    }
    double v[2] = {rd, rr};
    case_block_reduce<2>(v, 0u, pu_out, (size_t)G * k, k);
}

// r.d and r.r per case; beta = (r.d)_new / up; the new up, rr and iteration
// count; the stopping test (one block).  The flag raised here reaches
// any_flag only in k_mr_finish, after this iteration's k_mr_update2.
__global__ void __launch_bounds__(256) k_mr_beta(MState *st, const double *__restrict__ part, int G, int k, int limit)
{
    __shared__ double sh[256];
    __shared__ int s_any;
    if (st->any_flag) return;
    if (threadIdx.x == 0) s_any = 0;
    const double rd = case_sum_block(part, G, sh, k);
    const double rr = case_sum_block(part + (size_t)G * k, G, sh, k);
    const int j = threadIdx.x;
    if (j < k) {
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

// p = d + beta p for the active cases, with p's FP32 high and low parts
// (the tensor-core product's input) beside it
__global__ void __launch_bounds__(256)
k_mr_update2(int ns, int k, const MState *__restrict__ st, const double *__restrict__ D, double *__restrict__ P,
             float2 *__restrict__ Ps)
{
    if (st->any_flag) return;
    const int j = threadIdx.x % k;
    const double beta = st->beta[j];
    if (!st->active[j]) return;   // this thread's case is fixed
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)ns * k;
         t += (size_t)gridDim.x * blockDim.x) {
        const double pn = fma(P[t], beta, D[t]);
        P[t] = pn;
        float h, l;
        split_f64(pn, h, l);
        Ps[t] = make_float2(h, l);
    }
}

// Ps = FP32 high and low parts of P (block products outside a solve)
__global__ void k_mr_psplit(size_t n, const double *__restrict__ P, float2 *__restrict__ Ps)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        float h, l;
        split_f64(P[t], h, l);
        Ps[t] = make_float2(h, l);
    }
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
k_mr_replace(int ns, int k, const MState *__restrict__ st, const double *__restrict__ RRES,
             const double *__restrict__ dinv, double *__restrict__ R, double *__restrict__ D,
             double *__restrict__ part, int G)
{
    const int j = threadIdx.x % k;
    const bool act = st->active[j] != 0;
    double rd = 0.0, rr = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x, t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t ds = stride / k;   // the block size is a multiple of k
    size_t s = t0 / k;
    for (size_t t = t0; t < (size_t)ns * k; t += stride, s += ds) {
        if (!act) continue;
        const double rv = RRES[t], dv = dinv[s] * rv;
        R[t] = rv;
        D[t] = dv;
        rd = fma(rv, dv, rd);
        rr = fma(rv, rv, rr);
    }
    double v[2] = {rd, rr};
    case_block_reduce<2>(v, 0u, part, (size_t)G * k, k);
}

__global__ void k_mr_replace2(MState *st, const double *__restrict__ part, int G, int k)
{
    for (int j = threadIdx.x; j < k; j += blockDim.x)
        if (st->active[j]) {
            st->up[j] = case_sum(part, G, j, k);
            st->rr[j] = case_sum(part + (size_t)G * k, G, j, k);
            st->flag[j] = 0;
        }
    if (threadIdx.x == 0) {
        st->any_flag = 0;
        st->pending = 0;
    }
}

__global__ void k_mr_sums(const double *__restrict__ part, int G, int k, double *__restrict__ out)
{
    for (int j = threadIdx.x; j < k; j += blockDim.x) out[j] = case_sum(part, G, j, k);
}

__global__ void k_mr_eq_to_slot(int ns, int k, const int *__restrict__ slot_eq, int neq, const double *__restrict__ Req,
                                double *__restrict__ F)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)ns * k;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t s = t / k, j = t % k;
        const int q = slot_eq[s];
        F[t] = q > 0 ? Req[j * (size_t)neq + q - 1] : 0.0;
    }
}

__global__ void k_mr_slot_to_eq(int neq, int k, const int *__restrict__ eq_slot, const double *__restrict__ X,
                                double *__restrict__ Xeq)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)neq * k;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t j = t / neq, q = t % neq;
        Xeq[t] = X[(size_t)eq_slot[q] * k + j];
    }
}

// ---------------------------------------------------------------------------
// Block-solve buffers of one context (Ctx::multi), allocated on the first
// block solve or product and kept while the mesh and k are unchanged.
struct MultiBufs {
    int ns = 0, ne = 0, k = 0;
    double *F = nullptr, *X = nullptr, *R = nullptr, *D = nullptr, *P = nullptr, *U = nullptr, *RR = nullptr,
           *eq = nullptr;
    float *ut32 = nullptr;
    float2 *Ps = nullptr;           // [ns*k] FP32 high and low parts of P (the tensor-core product's input)
    unsigned char *rec = nullptr;   // [nels][kRecBytes] tensor-core element records
    double *ut64 = nullptr, *part = nullptr, *sums = nullptr;
    MState *st = nullptr;
    MState *hst = nullptr;
    // TMA maps of Ps for the tensor-core product's gathers: rows of one node
    // (box 3k x 1, passes over all k cases) and rows of one slot (box kb x 1
    // for kb = 8, 16, 32, 64); bit 0 / bit 1 + i set once encoded for Ps
    CUtensorMap tm_node;
    CUtensorMap tm_slot[4];
    unsigned tm_have = 0;
    // autotuned tensor-core pass width (cases per pass) for this k, and the
    // timings of the candidates (ms per full product)
    int kb = 0;
    int cand[4] = {0, 0, 0, 0};
    float cand_ms[4] = {0, 0, 0, 0};
};
namespace {
void mb_free_vectors(MultiBufs &m)
{
    void *p[] = {m.F, m.X, m.R, m.D, m.P, m.U, m.RR, m.eq, m.ut32, m.Ps, m.ut64, m.part, m.sums, m.st};
    for (void *q : p)
        if (q) cudaFree(q);
    if (m.hst) cudaFreeHost(m.hst);
    m.F = m.X = m.R = m.D = m.P = m.U = m.RR = m.eq = m.ut64 = m.part = m.sums = nullptr;
    m.ut32 = nullptr;
    m.Ps = nullptr;
    m.st = nullptr;
    m.hst = nullptr;
    m.ns = 0;
    m.k = 0;
    m.kb = 0;
    m.tm_have = 0;
}
void mb_free(MultiBufs &m)
{
    mb_free_vectors(m);
    if (m.rec) cudaFree(m.rec);
    m = MultiBufs();
}
}  // namespace

void multi_release(Ctx &c)
{
    if (!c.multi) return;
    mb_free(*c.multi);
    delete c.multi;
    c.multi = nullptr;
    c.mr_ok = false;
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

// record stages that fit the shared memory beside the P stages and tile sets
// for kb cases per pass (at most kMaxRec)
static int mr_stages(int kb)
{
    for (int nr = kMaxRec; nr >= 2; --nr)
        if (make_plan(kb, nr).smem <= 227 * 1024) return nr;
    return 0;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link the driver library itself)
static EncodeTiledFn encode_tiled()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

// A 2-D map of Ps (8-byte elements, rows of `cols` elements, `rows` rows),
// box `box` x 1: one gathered row per box.
static int mr_encode(CUtensorMap *tm, const float2 *Ps, int cols, size_t rows, int box)
{
    EncodeTiledFn fn = encode_tiled();
    if (!fn) {
        set_error("pf_solve_multi: cuTensorMapEncodeTiled is not available from the driver");
        return 1;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)cols * 8};
    const cuuint32_t boxd[2] = {(cuuint32_t)box, 1};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void *)Ps, dims, strides, boxd, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("pf_solve_multi: cuTensorMapEncodeTiled failed (%d) for %d x %zu, box %d", (int)r, cols, rows, box);
        return 1;
    }
    return 0;
}

template <int KB>
static int mr_tc_pass_t(Ctx &c, int c0, const int *skip)
{
    MultiBufs &m = *c.multi;
    const int whole = KB == m.k ? 1 : 0;
    constexpr int slot = KB == 64 ? 3 : KB == 32 ? 2 : KB == 16 ? 1 : 0;
    CUtensorMap *tm = whole ? &m.tm_node : &m.tm_slot[slot];
    const unsigned bit = whole ? 1u : 2u << slot;
    if (!(m.tm_have & bit)) {
        if (whole ? mr_encode(tm, m.Ps, 3 * m.k, (size_t)c.nn, 3 * KB)
                  : mr_encode(tm, m.Ps, m.k, (size_t)c.nslots, KB))
            return 1;
        m.tm_have |= bit;
    }
    const int nr = mr_stages(KB);
    const Plan pl = make_plan(KB, nr);
    static thread_local int attr_dev = -1;
    if (attr_dev != c.device) {
        MCK(cudaFuncSetAttribute(k_mr_elem_h16<KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        attr_dev = c.device;
    }
    const int grid = c.nels < c.nsm ? c.nels : c.nsm;
    k_mr_elem_h16<KB><<<grid, kH16Threads, pl.smem, c.stream>>>(c.nels, m.k, c0, nr, m.rec, c.conn, *tm, whole,
                                                               m.ut32, c.kerr, skip);
    return mr_launched(c, "k_mr_elem_h16");
}

// the tensor-core product of cases c0 .. c0+kb-1, kb in {8, 16, 32, 64}
// (input: the split P, m.Ps)
static int mr_tc_pass(Ctx &c, int kb, int c0, const int *skip)
{
    switch (kb) {
    case 64: return mr_tc_pass_t<64>(c, c0, skip);
    case 32: return mr_tc_pass_t<32>(c, c0, skip);
    case 16: return mr_tc_pass_t<16>(c, c0, skip);
    default: return mr_tc_pass_t<8>(c, c0, skip);
    }
}

// all k cases in passes of at most w cases: the widest of 64, 32, 16, 8 that
// fits the cases left (every k that is a multiple of 8 decomposes)
static int mr_tc_product(Ctx &c, int w, const int *skip)
{
    const int k = c.multi->k;
    for (int c0 = 0; c0 < k;) {
        int kb = 64;
        while (kb > w || kb > k - c0) kb >>= 1;
        if (mr_tc_pass(c, kb, c0, skip)) return 1;
        c0 += kb;
    }
    return 0;
}

// U = K P for the block (prec 16: tensor cores, on P's split copy m.Ps, which
// must hold P; 32: CUDA-core FP32, 64: FP64 into ut64).  skip: device flag
// that turns the launch into a no-op.
static int mr_elem(Ctx &c, int prec, const double *P, const int *skip)
{
    MultiBufs &m = *c.multi;
    if (prec == 16) return mr_tc_product(c, m.kb, skip);
    const int grid = (c.nels + 7) / 8 < c.nsm * 8 ? (c.nels + 7) / 8 : c.nsm * 8;
    if (prec == 32) {
        k_mr_elem_cc<float, float><<<grid, 256, 0, c.stream>>>(c.nels, m.k, c.km32, c.conn, P, m.ut32, skip);
        return mr_launched(c, "k_mr_elem_cc<float>");
    }
    k_mr_elem_cc<double, double><<<grid, 256, 0, c.stream>>>(c.nels, m.k, c.km64, c.conn, P, m.ut64, skip);
    return mr_launched(c, "k_mr_elem_cc<double>");
}

static int mr_scatter(Ctx &c, int prec, int mode, const double *pf, double *out, const int *skip)
{
    MultiBufs &m = *c.multi;
    const int G = c.Gs, T = case_threads(m.k);
    if (prec == 64) {
        if (mode == 0)
            k_mr_scatter<double, 0><<<G, T, 0, c.stream>>>(c.nn, m.k, c.node_ptr, c.node_list, m.ut64, c.freemask, pf,
                                                          out, m.part, skip);
        else
            k_mr_scatter<double, 1><<<G, T, 0, c.stream>>>(c.nn, m.k, c.node_ptr, c.node_list, m.ut64, c.freemask, pf,
                                                          out, m.part, skip);
    } else {
        if (mode == 0)
            k_mr_scatter<float, 0><<<G, T, 0, c.stream>>>(c.nn, m.k, c.node_ptr, c.node_list, m.ut32, c.freemask, pf,
                                                         out, m.part, skip);
        else
            k_mr_scatter<float, 1><<<G, T, 0, c.stream>>>(c.nn, m.k, c.node_ptr, c.node_list, m.ut32, c.freemask, pf,
                                                         out, m.part, skip);
    }
    return mr_launched(c, "k_mr_scatter");
}

static int mr_alloc(Ctx &c, int k)
{
    if (!c.multi) c.multi = new MultiBufs();
    MultiBufs &m = *c.multi;
    if (m.ne != c.nels) {
        mb_free(m);
        c.mr_ok = false;
    }
    if (!m.rec && cudaMalloc((void **)&m.rec, (size_t)c.nels * kRecBytes) != cudaSuccess) {
        set_error("pf_solve_multi: cannot allocate the tensor-core element records (%zu bytes)",
                  (size_t)c.nels * kRecBytes);
        return 1;
    }
    m.ne = c.nels;
    if (m.ns == c.nslots && m.k == k && m.F) return 0;
    mb_free_vectors(m);
    const size_t n = (size_t)c.nslots * k;
    const size_t parts = (size_t)(c.Gs > c.G ? c.Gs : c.G) * k * 4 + 64;
    double **v[] = {&m.F, &m.X, &m.R, &m.D, &m.P, &m.U, &m.RR};
    for (double **q : v)
        if (cudaMalloc((void **)q, n * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.eq, (size_t)(c.neq > 0 ? c.neq : 1) * k * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.ut32, (size_t)c.nels * 60 * k * 4) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.Ps, n * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.ut64, (size_t)c.nels * 60 * k * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.part, parts * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.sums, kMaxK * 8) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&m.st, sizeof(MState)) != cudaSuccess) goto fail;
    if (cudaMallocHost((void **)&m.hst, sizeof(MState)) != cudaSuccess) goto fail;
    m.ns = c.nslots;
    m.k = k;
    return 0;
fail:
    mb_free_vectors(m);
    set_error("pf_solve_multi: cannot allocate the block vectors (%zu slots x %d cases)", (size_t)c.nslots, k);
    return 1;
}

// The element records of the tensor-core product (when storkm changed), and
// the widest pass for this k: each candidate (the three widest of 64, 32,
// 16, 8 that do not exceed k) times one full product (after one untimed),
// the fastest is kept.  The candidates differ only in how many cases one
// pass carries; each case's operands, scales and products are formed the
// same way.
static int mr_prepare_tc(Ctx &c)
{
    MultiBufs &m = *c.multi;
    if (!c.mr_ok) {
        k_mr_pack<<<c.nsm * 16, 128, 0, c.stream>>>(c.nels, c.km64, m.rec);
        if (mr_launched(c, "k_mr_pack")) return 1;
        c.mr_ok = true;
        m.kb = 0;
    }
    if (m.kb) return 0;
    const int k = m.k;
    int n = 0;
    for (int w : {64, 32, 16, 8})
        if (w <= k && n < 3) m.cand[n++] = w;
    for (int i = n; i < 4; ++i) m.cand[i] = 0, m.cand_ms[i] = 0.f;
    if (n == 1) {
        m.kb = m.cand[0];
        m.cand_ms[0] = 0.f;
        return 0;
    }
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        set_error("multi-RHS autotune: cannot create events");
        return 1;
    }
    float best = 1e30f;
    for (int i = 0; i < n; ++i) {
        if (mr_tc_product(c, m.cand[i], nullptr)) return 1;
        cudaEventRecord(a, c.stream);
        if (mr_tc_product(c, m.cand[i], nullptr)) return 1;
        cudaEventRecord(b, c.stream);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        m.cand_ms[i] = ms;
        if (ms < best) {
            best = ms;
            m.kb = m.cand[i];
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return 0;
}

// FP64 true residuals of all cases; returns per-case ||f - K x||^2 in rr_out
static int mr_true_residual(Ctx &c, double *rr_out)
{
    MultiBufs &m = *c.multi;
    if (mr_elem(c, 64, m.X, nullptr)) return 1;
    if (mr_scatter(c, 64, 1, m.F, m.RR, nullptr)) return 1;
    k_mr_sums<<<1, 128, 0, c.stream>>>(m.part, c.Gs, m.k, m.sums);
    if (mr_launched(c, "k_mr_sums")) return 1;
    MCK(cudaMemcpyAsync(rr_out, m.sums, m.k * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    MCK(cudaStreamSynchronize(c.stream));
    return 0;
}

static int mr_check_k(const char *who, int k)
{
    if (k < 8 || k > kMaxK || k % 8) {
        set_error("%s: k must be a multiple of 8 in 8..%d (got %d)", who, kMaxK, k);
        return 1;
    }
    return 0;
}

static int mr_kernel_error(Ctx &c, const char *who)
{
    int kerr = 0;
    MCK(cudaMemcpy(&kerr, c.kerr, sizeof(int), cudaMemcpyDeviceToHost));
    if (kerr) {
        cudaMemset(c.kerr, 0, sizeof(int));
        set_error("%s: tensor-core product wait timed out", who);
        return 1;
    }
    return 0;
}

extern "C" int pf_solve_multi(void **ctx, const int *k_p, const double *r, const double *tol, const int *limit,
                              const int *prec, double *xnew, int *iters, double *relres)
try {
    if (!ctx || !*ctx || !k_p || !r || !tol || !limit || !prec || !xnew || !iters || !relres) {
        set_error("pf_solve_multi: null argument");
        return PF_FAILURE;
    }
    Ctx &c = *(Ctx *)*ctx;
    MCK(cudaSetDevice(c.device));
    if (mr_check_k("pf_solve_multi", *k_p)) return PF_FAILURE;
    const int k = *k_p;
    if (c.shared || c.kind != KIND_SOLID20) {
        set_error("pf_solve_multi: needs per-element 20-node storkm");
        return PF_FAILURE;
    }
    if (!c.have_km || *limit < 1 || (*prec != 16 && *prec != 32)) {
        set_error("pf_solve_multi: needs storkm, limit >= 1 and prec 16 (tensor cores) or 32 (CUDA cores)");
        return PF_FAILURE;
    }
    if (mr_alloc(c, k)) return PF_FAILURE;
    MultiBufs &m = *c.multi;
    const int G = c.G, Gs = c.Gs, T = case_threads(k);
    // load cases: r(neq, k) column-major
    MCK(cudaMemcpyAsync(m.eq, r, (size_t)c.neq * k * 8, cudaMemcpyHostToDevice, c.stream));
    k_mr_eq_to_slot<<<c.nsm * 8, 256, 0, c.stream>>>(c.nslots, k, c.slot_eq, c.neq, m.eq, m.F);
    if (mr_launched(c, "k_mr_eq_to_slot")) return PF_FAILURE;
    if (*prec == 16) {
        // the autotuner times products of the initial search directions
        k_mr_init<<<G, T, 0, c.stream>>>(c.nslots, k, m.F, c.dinv, m.X, m.R, m.D, m.P, m.Ps, m.part, G);
        if (mr_launched(c, "k_mr_init")) return PF_FAILURE;
        if (mr_prepare_tc(c)) return PF_FAILURE;
    }
    cudaEvent_t e0, e1;
    MCK(cudaEventCreate(&e0));
    MCK(cudaEventCreate(&e1));
    MCK(cudaEventRecord(e0, c.stream));
    k_mr_init<<<G, T, 0, c.stream>>>(c.nslots, k, m.F, c.dinv, m.X, m.R, m.D, m.P, m.Ps, m.part, G);
    if (mr_launched(c, "k_mr_init")) return PF_FAILURE;
    k_mr_init2<<<1, 128, 0, c.stream>>>(m.st, m.part, G, k, *tol);
    if (mr_launched(c, "k_mr_init2")) return PF_FAILURE;
    double *pu = m.part + (size_t)Gs * k;   // update partials after the scatter partials
    int total = 0, chunk = 4, corrections = 0;
    std::vector<double> rel(k, 0.0), rr(k, 0.0);
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
            k_mr_alpha<<<1, 256, 0, c.stream>>>(m.st, m.part, Gs, k);
            if (mr_launched(c, "k_mr_alpha")) return PF_FAILURE;
            k_mr_update1<<<G, T, 0, c.stream>>>(c.nslots, k, m.st, pu, G, m.X, m.R, m.D, m.P, m.U, c.dinv);
            if (mr_launched(c, "k_mr_update1")) return PF_FAILURE;
            k_mr_beta<<<1, 256, 0, c.stream>>>(m.st, pu, G, k, *limit);
            if (mr_launched(c, "k_mr_beta")) return PF_FAILURE;
            k_mr_update2<<<G, T, 0, c.stream>>>(c.nslots, k, m.st, m.D, m.P, m.Ps);
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
        if (mr_kernel_error(c, "pf_solve_multi")) return PF_FAILURE;
        if (m.hst->err) {
            set_error("pf_solve_multi: PCG breakdown (non-finite r.d)");
            return PF_FAILURE;
        }
        if (!m.hst->any_flag) continue;
        // some active case reached its threshold (or the limit): FP64 true residuals
        if (mr_true_residual(c, rr.data())) return PF_FAILURE;
        int n_active = 0;
        for (int j = 0; j < k; ++j) {
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
        k_mr_replace<<<G, T, 0, c.stream>>>(c.nslots, k, m.st, m.RR, c.dinv, m.R, m.D, m.part, G);
        if (mr_launched(c, "k_mr_replace")) return PF_FAILURE;
        k_mr_replace2<<<1, 128, 0, c.stream>>>(m.st, m.part, G, k);
        if (mr_launched(c, "k_mr_replace2")) return PF_FAILURE;
        ++corrections;
        chunk = 4;
    }
    for (auto &ev : tev) cudaEventDestroy(ev);
    MCK(cudaEventRecord(e1, c.stream));
    k_mr_slot_to_eq<<<c.nsm * 8, 256, 0, c.stream>>>(c.neq, k, c.eq_slot, m.X, m.eq);
    if (mr_launched(c, "k_mr_slot_to_eq")) return PF_FAILURE;
    MCK(cudaMemcpyAsync(xnew, m.eq, (size_t)c.neq * k * 8, cudaMemcpyDeviceToHost, c.stream));
    MCK(cudaStreamSynchronize(c.stream));
    float ms = 0.f;
    MCK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int j = 0; j < k; ++j) {
        iters[j] = m.hst->iters[j];
        relres[j] = rel[j];
    }
    c.stats[0] = 0;
    for (int j = 0; j < k; ++j) c.stats[0] = iters[j] > c.stats[0] ? iters[j] : c.stats[0];
    c.stats[1] = corrections;
    c.stats[2] = ms;
    c.stats[3] = ms_elem;   // summed element-product time of the launched iterations
    c.stats[4] = ms_scat;   // summed scatter time
    c.stats[5] = ms_iter;   // summed time of the iterations measured start to start
    c.stats[6] = total;     // iterations launched (including no-op ones after a flag)
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_solve_multi");
}

// Block product U = K P for k cases in equation order (tests): prec 16, 32
// or 64.
extern "C" int pf_ebe_matvec_multi(void **ctx, const int *k_p, const int *prec, const double *p, double *u)
try {
    if (!ctx || !*ctx || !k_p || !prec || !p || !u) {
        set_error("pf_ebe_matvec_multi: null argument");
        return PF_FAILURE;
    }
    Ctx &c = *(Ctx *)*ctx;
    MCK(cudaSetDevice(c.device));
    if (mr_check_k("pf_ebe_matvec_multi", *k_p)) return PF_FAILURE;
    const int k = *k_p;
    if (!c.have_km || c.shared || c.kind != KIND_SOLID20 || (*prec != 16 && *prec != 32 && *prec != 64)) {
        set_error("pf_ebe_matvec_multi: prec 16/32/64 and per-element storkm formed");
        return PF_FAILURE;
    }
    if (mr_alloc(c, k)) return PF_FAILURE;
    MultiBufs &m = *c.multi;
    MCK(cudaMemcpyAsync(m.eq, p, (size_t)c.neq * k * 8, cudaMemcpyHostToDevice, c.stream));
    k_mr_eq_to_slot<<<c.nsm * 8, 256, 0, c.stream>>>(c.nslots, k, c.slot_eq, c.neq, m.eq, m.P);
    if (mr_launched(c, "k_mr_eq_to_slot")) return PF_FAILURE;
    if (*prec == 16) {
        k_mr_psplit<<<c.nsm * 8, 256, 0, c.stream>>>((size_t)c.nslots * k, m.P, m.Ps);
        if (mr_launched(c, "k_mr_psplit")) return PF_FAILURE;
        if (mr_prepare_tc(c)) return PF_FAILURE;
    }
    if (mr_elem(c, *prec, m.P, nullptr)) return PF_FAILURE;
    if (mr_scatter(c, *prec, 0, m.P, m.U, nullptr)) return PF_FAILURE;
    k_mr_slot_to_eq<<<c.nsm * 8, 256, 0, c.stream>>>(c.neq, k, c.eq_slot, m.U, m.eq);
    if (mr_launched(c, "k_mr_slot_to_eq")) return PF_FAILURE;
    MCK(cudaMemcpyAsync(u, m.eq, (size_t)c.neq * k * 8, cudaMemcpyDeviceToHost, c.stream));
    MCK(cudaStreamSynchronize(c.stream));
    if (mr_kernel_error(c, "pf_ebe_matvec_multi")) return PF_FAILURE;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_ebe_matvec_multi");
}

extern "C" int pf_multi_product_ms(void **ctx, const int *k_p, const double *p, const int *reps, double *ms)
try {
    if (!ctx || !*ctx || !k_p || !p || !reps || !ms || *reps < 1) {
        set_error("pf_multi_product_ms: null argument or reps < 1");
        return PF_FAILURE;
    }
    Ctx &c = *(Ctx *)*ctx;
    MCK(cudaSetDevice(c.device));
    if (mr_check_k("pf_multi_product_ms", *k_p)) return PF_FAILURE;
    const int k = *k_p;
    if (!c.have_km || c.shared || c.kind != KIND_SOLID20) {
        set_error("pf_multi_product_ms: needs per-element 20-node storkm");
        return PF_FAILURE;
    }
    if (mr_alloc(c, k)) return PF_FAILURE;
    MultiBufs &m = *c.multi;
    MCK(cudaMemcpyAsync(m.eq, p, (size_t)c.neq * k * 8, cudaMemcpyHostToDevice, c.stream));
    k_mr_eq_to_slot<<<c.nsm * 8, 256, 0, c.stream>>>(c.nslots, k, c.slot_eq, c.neq, m.eq, m.P);
    if (mr_launched(c, "k_mr_eq_to_slot")) return PF_FAILURE;
    k_mr_psplit<<<c.nsm * 8, 256, 0, c.stream>>>((size_t)c.nslots * k, m.P, m.Ps);
    if (mr_launched(c, "k_mr_psplit")) return PF_FAILURE;
    if (mr_prepare_tc(c)) return PF_FAILURE;
    if (mr_tc_product(c, m.kb, nullptr)) return PF_FAILURE;   // warm-up
    cudaEvent_t a, b;
    MCK(cudaEventCreate(&a));
    MCK(cudaEventCreate(&b));
    MCK(cudaEventRecord(a, c.stream));
    for (int r = 0; r < *reps; ++r)
        if (mr_tc_product(c, m.kb, nullptr)) return PF_FAILURE;
    MCK(cudaEventRecord(b, c.stream));
    MCK(cudaEventSynchronize(b));
    float t = 0.f;
    MCK(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (mr_kernel_error(c, "pf_multi_product_ms")) return PF_FAILURE;
    *ms = t / *reps;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_multi_product_ms");
}

extern "C" int pf_multi_tuning(void **ctx, int *kb, int *cand, float *ms)
try {
    if (!ctx || !*ctx || !kb || !cand || !ms) {
        set_error("pf_multi_tuning: null argument");
        return PF_FAILURE;
    }
    Ctx &c = *(Ctx *)*ctx;
    if (!c.multi || !c.multi->kb) {
        set_error("pf_multi_tuning: no tensor-core block product has run on this context");
        return PF_FAILURE;
    }
    *kb = c.multi->kb;
    for (int i = 0; i < 4; ++i) {
        cand[i] = c.multi->cand[i];
        ms[i] = c.multi->cand_ms[i];
    }
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_multi_tuning");
}

extern "C" int pf_multi_free(void **ctx)
try {
    if (!ctx || !*ctx) return PF_SUCCESS;
    Ctx &c = *(Ctx *)*ctx;
    cudaSetDevice(c.device);
    cudaStreamSynchronize(c.stream);
    multi_release(c);
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_multi_free");
}
