// pf_shared.cu -- element products when every element has the same
// stiffness matrix km (PCG_KM, src/modules/mpi/maths.f90:1152-1323, whose
// iteration computes utemp = MATMUL(km, pmul) over all elements at once;
// the uniform-mesh GPU experiment xx9, src/programs/dev/xx9/mathsgpu.f90).
//
// With one km the product is a true GEMM, U(60 x nels) = km(60 x 60) *
// P(60 x nels), and no per-element matrix is streamed from HBM.
//   k_elem_shared64   FP64 on CUDA cores: km in shared memory, one warp per
//                     element (bound by FP64 FMA throughput, as k_elem<double>).
//   k_elem_shared_tc  FP32-class on the tensor cores: km split once into
//                     three BF16 terms held in shared memory for the whole
//                     kernel; tiles of 128 elements' gathered p values are
//                     split the same way; the six products of order <= 2^-16
//                     accumulate in FP32 in TMEM (M = 128: km's rows in four
//                     blocks of five nodes, each block with the three
//                     direction sums of km's rows; N = 128 elements,
//                     K = 64).  The product is P km P p_e, P removing the
//                     element's mean translation, as in the packed per-element
//                     kernel.  Warp-specialised:
//                     connectivity copies, gather + split, MMA issue and the
//                     TMEM read-back overlap across tiles through mbarrier
//                     rings.  Results are written in the node-padded FP32
//                     layout the scatter reads.
#include "pf_device.cuh"
#include "pf_tc.cuh"

namespace pf {

using namespace tc;

namespace {

constexpr int kNT = 128;                    // elements per tile (MMA N)
constexpr int kSRowsA = 128;                // A rows: 4 blocks of 32 (15 node rows, 3 sum rows, 14 zero rows)
constexpr int kSTermA = kSRowsA * 64 * 2;   // 16 KB: one km term, K = 64
constexpr int kSBufA = 3 * kSTermA;
constexpr int kSTermB = kNT * 64 * 2;       // 16 KB: 128 elements x 64 K
constexpr int kSBufB = 3 * kSTermB;
constexpr int kSConn = kNT * 20 * 4;        // 10 KB: connectivity of one tile
constexpr int kSNB = 3;                     // B tile sets in flight
constexpr int kSNC = 3;                     // connectivity buffers in flight
constexpr int kSNA = 4;                     // TMEM accumulators (128 columns each, all 512)
constexpr int kSGather = 16;                // warps 0-15 gather p and split it (two tasks per thread)
constexpr int kSEpi0 = 16;                  // warps 16-19 read TMEM lanes 32w..32w+31 back, five nodes each
constexpr int kSNEpi = 4;
constexpr int kSProd = 20;                  // warp 20 copies the connectivity
constexpr int kSMma = 21;                   // warp 21, lane 0 issues the MMAs
constexpr int kSThreads = 22 * 32;
constexpr int kSOffB = kSBufA;
constexpr int kSOffC = kSOffB + kSNB * kSBufB;
constexpr int kSOffAux = kSOffC + kSNC * kSConn;
constexpr int kSSmem = kSOffAux + 256;
constexpr uint32_t kSIdesc = idesc_bf16(128, kNT);
static_assert(kSOffC % 16 == 0 && kSConn % 16 == 0 && kSOffAux % 8 == 0, "bulk-copy alignment");
static_assert(kSSmem <= 227 * 1024, "shared memory per CTA");
static_assert(kSGather * 32 * 2 == kNT * 8, "two B tasks (element, 8 dofs) per gather thread");
static_assert(kSEpi0 % 4 == 0, "epilogue warp kSEpi0 + w must reach TMEM lanes 32w..32w+31");

__device__ __forceinline__ void mbar_arrive1(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

}  // namespace

// u_e = km p_e in FP64 for every element (results utemp[e*60 + i]).
__global__ void __launch_bounds__(256)
k_elem_shared64(int nels, const double *__restrict__ km, const int *__restrict__ conn,
                const double *__restrict__ p, double *__restrict__ ut, const PcgState *__restrict__ st)
{
    __shared__ __align__(16) double ks[3600];
    if (block_stopped(st)) return;
    for (int i = threadIdx.x; i < 3600; i += blockDim.x) ks[i] = km[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int j1 = lane + 32;
    for (int e = warp; e < nels; e += nwarps) {
        const int nd = (lane < 20) ? conn[(size_t)e * 20 + lane] : 0;
        const int n0 = __shfl_sync(FULLMASK, nd, lane / 3);
        const int n1 = __shfl_sync(FULLMASK, nd, j1 < 60 ? j1 / 3 : 0);
        const double p0 = p[(size_t)3 * n0 + lane % 3];
        const double p1 = (j1 < 60) ? p[(size_t)3 * n1 + j1 % 3] : 0.0;
        double a0 = 0.0, a1 = 0.0;
#pragma unroll 12
        for (int j = 0; j < 60; ++j) {   // ascending column order, as k_elem<double>
            const double pj = __shfl_sync(FULLMASK, j < 32 ? p0 : p1, j & 31);
            if (lane < 30) {
                const double2 k2 = *reinterpret_cast<const double2 *>(ks + 60 * j + 2 * lane);
                a0 = fma(k2.x, pj, a0);
                a1 = fma(k2.y, pj, a1);
            }
        }
        if (lane < 30) reinterpret_cast<double2 *>(ut + (size_t)e * 60)[lane] = make_double2(a0, a1);
    }
}

// u_e = P km P p_e on the tensor cores for every element (FP32 results,
// node-padded: row i of element e at e*80 + (i/3)*4 + i%3).
// One persistent CTA of 22 warps per SM walks the tiles T = blockIdx.x +
// t * gridDim.x with warp-specialised roles linked by mbarriers:
//   warp 20      bulk-copies each tile's connectivity into a ring of kSNC;
//   warps 0-15   gather the tile's p values (two 8-dof tasks per thread),
//                remove each element's mean translation, split the values
//                into three BF16 terms and write a ring of kSNB B tile sets;
//   warp 21      one thread issues the six products (24 MMAs, M=128, N=128,
//                K=16) into a ring of kSNA TMEM accumulators;
//   warps 16-19  read TMEM lanes 0..127 back (five nodes each), remove
//                each element's mean translation and store the results.
// Every wait is bounded.  A wait that runs out sets a shared failure flag
// that every role checks before its next wait, writes 3 to the device error
// word, and the CTA waits (bounded) for the copies and MMAs it has in flight
// before it frees its TMEM and returns.
__global__ void __launch_bounds__(kSThreads, 1)
k_elem_shared_tc(int nels, const float *__restrict__ km32, const int *__restrict__ conn,
                 const float2 *__restrict__ ps, float *__restrict__ ut, const PcgState *__restrict__ st,
                 int *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *A = sm;
    unsigned char *B = sm + kSOffB;
    int *cs = reinterpret_cast<int *>(sm + kSOffC);                   // [kSNC][128*20]
    uint64_t *c_full = reinterpret_cast<uint64_t *>(sm + kSOffAux);
    uint64_t *c_empty = c_full + kSNC;
    uint64_t *b_full = c_empty + kSNC;
    uint64_t *b_empty = b_full + kSNB;
    uint64_t *a_full = b_empty + kSNB;
    uint64_t *a_empty = a_full + kSNA;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(a_empty + kSNA);
    volatile int *s_fail = reinterpret_cast<volatile int *>(tslot + 1);
    int *s_count = reinterpret_cast<int *>(tslot + 2);   // [0] copies issued, [1] MMA groups committed
    int *s_stop = s_count + 2;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) *s_stop = st ? st->stop : 0;
    __syncthreads();
    if (*s_stop) return;   // uniform: read once per block
    const int ntiles = (nels + kNT - 1) / kNT;
    const int nmine = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto tile = [&](int t) { return (int)blockIdx.x + t * (int)gridDim.x; };
    auto tile_n = [&](int t) { const int r = nels - tile(t) * kNT; return r < kNT ? r : kNT; };

    // km once, three BF16 terms.  A row 32w + i is K row 3(5w + i/3) + i%3
    // for i < 15 (nodes 5w..5w+4), the sum of K's 20 rows of direction
    // i - 15 for i = 15..17, zero otherwise.  The sums are zero in exact
    // arithmetic (K annihilates rigid translations); they carry the rounding
    // of the FP32 km and put each element's per-direction sum of results
    // beside its rows in the accumulator.  K(i,k) = km32[i + 60k]; the sums
    // follow km (km32[3600 + 64d + k]), so the prologue has no FP64 work.
    for (int i = tid; i < kSOffC / 16; i += kSThreads) reinterpret_cast<uint4 *>(sm)[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    for (int task = tid; task < kSRowsA * 8; task += kSThreads) {
        const int row = task % kSRowsA, q = task / kSRowsA;
        const int w = row >> 5, i = row & 31;
        float xv[8];
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const int k = 8 * q + g;
            float v = 0.f;
            if (k < 60 && i < 15) {
                v = km32[3 * (5 * w + i / 3) + i % 3 + 60 * k];
            } else if (k < 60 && i < 18) {
                v = km32[3600 + 64 * (i - 15) + k];   // formed on the host with km
            }
            xv[g] = v;
        }
        split3_store8(xv, A + kmajor_off(row, 8 * q), kSTermA);
    }
    if (warp == 0) tmem_alloc(tslot, 512);
    if (tid == 0) {
        for (int i = 0; i < kSNC; ++i) {
            mbar_init(&c_full[i], 1);
            mbar_init(&c_empty[i], kSGather);
        }
        for (int i = 0; i < kSNB; ++i) {
            mbar_init(&b_full[i], kSGather);
            mbar_init(&b_empty[i], 1);
        }
        for (int i = 0; i < kSNA; ++i) {
            mbar_init(&a_full[i], 1);
            mbar_init(&a_empty[i], kSNEpi);
        }
        mbar_fence_init();
        *s_fail = 0;
        s_count[0] = s_count[1] = 0;
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

    if (warp == kSProd) {
        int t = 0;
        if (lane == 0) {
            for (; t < nmine; ++t) {
                const int b = t % kSNC;
                if (t >= kSNC && !wait(&c_empty[b], (uint32_t)((t / kSNC - 1) & 1))) break;
                const uint32_t bytes = (uint32_t)tile_n(t) * 80u;
                mbar_expect_tx(&c_full[b], bytes);
                bulk_g2s(cs + b * kNT * 20, conn + (size_t)tile(t) * kNT * 20, bytes, &c_full[b]);
            }
            s_count[0] = t;
        }
        __syncwarp();
    } else if (warp < kSGather) {
        for (int t = 0; t < nmine; ++t) {
            const int cb = t % kSNC, bb = t % kSNB;
            if (!wait(&c_full[cb], (uint32_t)((t / kSNC) & 1))) break;
            if (t >= kSNB && !wait(&b_empty[bb], (uint32_t)((t / kSNB - 1) & 1))) break;
            const int *ct = cs + cb * kNT * 20;
            const int n_here = tile_n(t);
            // Lane j + 4 qq of warp w holds dofs 8qq..8qq+7 of elements
            // 8w + j (pass 0) and 8w + 4 + j (pass 1), so an element's eight
            // chunks are the lanes j, j+4, ..., j+28.  Each element's mean
            // translation is removed before the BF16 split (K t = 0 for a
            // rigid translation t, so the product is unchanged in exact
            // arithmetic and the rounding acts only on p - t).
            const int j = lane & 3, qq = lane >> 2;
            const int r = (2 * qq) % 3;   // direction of dof 8qq; dof 8qq+g has (r + g) % 3
            float2 pv[2][8];   // p's FP32 high and low parts; both passes' loads in flight together
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int n = 8 * warp + 4 * h + j;
#pragma unroll
                for (int g = 0; g < 8; ++g) {
                    const int c = 8 * qq + g;
                    pv[h][g] = (c < 60 && n < n_here) ? ps[(size_t)3 * ct[n * 20 + c / 3] + c % 3] : make_float2(0.f, 0.f);
                }
            }
            float xv[2][8];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float hi[8], lo[8];
#pragma unroll
                for (int g = 0; g < 8; ++g) {
                    hi[g] = pv[h][g].x;
                    lo[g] = pv[h][g].y;
                }
                // sums of this chunk by direction, then over the element's chunks
                const float u0 = hi[0] + hi[3] + hi[6], u1 = hi[1] + hi[4] + hi[7], u2 = hi[2] + hi[5];
                float s0 = r == 0 ? u0 : r == 1 ? u2 : u1;
                float s1 = r == 0 ? u1 : r == 1 ? u0 : u2;
                float s2 = r == 0 ? u2 : r == 1 ? u1 : u0;
#pragma unroll
                for (int o = 4; o < 32; o <<= 1) {
                    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
                    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
                    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
                }
                const float t0 = 0.05f * s0, t1 = 0.05f * s1, t2 = 0.05f * s2;
                const float tr[3] = {r == 0 ? t0 : r == 1 ? t1 : t2, r == 0 ? t1 : r == 1 ? t2 : t0,
                                     r == 0 ? t2 : r == 1 ? t0 : t1};
#pragma unroll
                for (int g = 0; g < 8; ++g) xv[h][g] = (8 * qq + g < 60) ? (hi[g] - tr[g % 3]) + lo[g] : 0.f;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive1(&c_empty[cb]);   // connectivity read
            unsigned char *Bb = B + bb * kSBufB;
            // even chunks store pass 0 first, odd chunks pass 1: each quarter
            // warp then writes eight different 16-byte bank groups
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int h = (qq & 1) ^ k;
                float y[8];
#pragma unroll
                for (int g = 0; g < 8; ++g) y[g] = h ? xv[1][g] : xv[0][g];
                split3_store8(y, Bb + kmajor_off(8 * warp + 4 * h + j, 8 * qq), kSTermB);
            }
            fence_proxy_async();   // this thread's tile writes -> the tensor cores
            __syncwarp();
            if (lane == 0) mbar_arrive1(&b_full[bb]);
        }
    } else if (warp == kSMma) {
        int t = 0;
        if (lane == 0) {
            for (; t < nmine; ++t) {
                const int bb = t % kSNB, a = t % kSNA;
                if (!wait(&b_full[bb], (uint32_t)((t / kSNB) & 1))) break;
                if (t >= kSNA && !wait(&a_empty[a], (uint32_t)((t / kSNA - 1) & 1))) break;
                tc_fence_after();
                const uint32_t b0 = smem_u32(B + bb * kSBufB), a0 = smem_u32(A);
                // the six products of order <= 2^-16: (1,1) (1,2) (2,1) (1,3) (2,2) (3,1)
                const int ta[6] = {0, 0, 1, 0, 1, 2};
                const int tb[6] = {0, 1, 0, 2, 1, 0};
                uint32_t acc = 0;
#pragma unroll
                for (int tt = 0; tt < 6; ++tt)
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks) {
                        mma_bf16(tmem + (uint32_t)(a * kNT), umma_desc(a0 + ta[tt] * kSTermA + ks * 256, 128, 1024),
                                 umma_desc(b0 + tb[tt] * kSTermB + ks * 256, 128, 1024), kSIdesc, acc);
                        acc = 1;
                    }
                mma_commit(&b_empty[bb]);
                mma_commit(&a_full[a]);
            }
            s_count[1] = t;
        }
        __syncwarp();
    } else if (warp >= kSEpi0 && warp < kSEpi0 + kSNEpi) {
        // TMEM lanes 32w + i: i < 15 row 3(5w + i/3) + i%3, i = 15..17 the
        // sums of direction i - 15.  Subtracting a twentieth of the sum of
        // the row's direction removes the result's mean translation (u_e =
        // P km P p_e); the five nodes' results are 80 contiguous bytes.
        const int w = warp - kSEpi0;
        const int src = lane < 15 ? 15 + lane % 3 : lane;
        // lanes 0..14 write the five nodes' 15 results, lanes 15..19 their
        // padding words, so every 32-byte sector of the results is written
        // whole (a partly written sector costs L2 a read of it from DRAM:
        // 300 MB of reads per launch at 100^3 without the padding words)
        const int roff = lane < 15 ? (5 * w + lane / 3) * 4 + lane % 3 : (5 * w + lane - 15) * 4 + 3;
        for (int t = 0; t < nmine; ++t) {
            const int a = t % kSNA;
            if (!wait(&a_full[a], (uint32_t)((t / kSNA) & 1))) break;
            tc_fence_after();
            const int n_here = tile_n(t);
            const size_t e0 = (size_t)tile(t) * kNT;
#pragma unroll 1
            for (int ch = 0; ch < kNT / 32; ++ch) {   // 32 columns per TMEM round trip
                float v[32];
                tmem_ld_32x32b_x32(tmem + ((uint32_t)(32 * w) << 16) + (uint32_t)(a * kNT + 32 * ch), v);
#pragma unroll
                for (int x = 0; x < 32; ++x) v[x] -= 0.05f * __shfl_sync(0xffffffffu, v[x], src);
                if (lane < 20) {
#pragma unroll
                    for (int x = 0; x < 32; ++x) {
                        const int n = 32 * ch + x;
                        if (n < n_here) ut[(e0 + n) * 80 + roff] = lane < 15 ? v[x] : 0.f;
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive1(&a_empty[a]);
        }
    }
    __syncthreads();
    if (*s_fail) {
        if (tid == 0) {
            atomicExch(err, 3);
            for (int t = s_count[0] - kSNC; t < s_count[0]; ++t)
                if (t >= 0) mbar_wait(&c_full[t % kSNC], (uint32_t)((t / kSNC) & 1));
            for (int t = s_count[1] - kSNA; t < s_count[1]; ++t)
                if (t >= 0) mbar_wait(&a_full[t % kSNA], (uint32_t)((t / kSNA) & 1));
        }
        __syncthreads();
    }
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// ediag[e*60 + i] = km(i,i) for every element
__global__ void k_shared_ediag(int nels, const double *__restrict__ km, double *__restrict__ ediag)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)nels * 60;
         t += (size_t)gridDim.x * blockDim.x)
        ediag[t] = km[(t % 60) * 61];
}

int launch_shared_ediag(Ctx &c)
{
    k_shared_ediag<<<c.nsm * 8, 256, 0, c.stream>>>(c.nels, c.skm64, c.ediag);
    c.launches++;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("k_shared_ediag: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

// u_e = km p_e for every element: prec 64 on CUDA cores in FP64, otherwise
// on the tensor cores (FP32-class).  st: PCG state whose stop flag turns the
// launch into a no-op (nullptr outside a PCG run).
// ps[s] = FP32 high and low parts of p[s]
__global__ void k_split_p(int ns, const double *__restrict__ p, float2 *__restrict__ ps)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        float h, l;
        split_f64(p[s], h, l);
        ps[s] = make_float2(h, l);
    }
}

int launch_elem_shared(Ctx &c, int prec, const double *p, const PcgState *st)
{
    cudaError_t e;
    if (prec == PREC_FP64) {
        long long g = ((long long)c.nels + 7) / 8;
        if (g > (long long)c.nsm * 8) g = (long long)c.nsm * 8;
        if (g < 1) g = 1;
        k_elem_shared64<<<(int)g, 256, 0, c.stream>>>(c.nels, c.skm64, c.conn, p, (double *)c.utemp, st);
    } else {
        if (!c.shared_attr) {   // set once, before any stream capture
            e = cudaFuncSetAttribute(k_elem_shared_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSSmem);
            if (e != cudaSuccess) {
                set_error("k_elem_shared_tc: cannot reserve %d bytes of shared memory: %s", kSSmem,
                          cudaGetErrorString(e));
                return 1;
            }
            c.shared_attr = true;
        }
        // the kernel gathers p's FP32 high and low parts: the PCG kernels
        // keep them with c.p; any other vector is split here first
        if (p != c.p) {
            k_split_p<<<c.nsm * 8, 256, 0, c.stream>>>(c.nslots, p, c.psplit);
            c.launches++;
        }
        const int ntiles = (c.nels + kNT - 1) / kNT;
        const int grid = ntiles < c.nsm ? ntiles : c.nsm;
        k_elem_shared_tc<<<grid, kSThreads, kSSmem, c.stream>>>(c.nels, c.skm32, c.conn, c.psplit, (float *)c.utemp,
                                                                 st, c.kerr);
    }
    c.launches++;
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("shared-km element product: launch failed: %s", cudaGetErrorString(e));
        return 1;
    }
    return 0;
}

}  // namespace pf
