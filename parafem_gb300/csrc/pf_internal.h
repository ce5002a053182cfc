// pf_internal.h -- device state of one solver context and the kernel entry
// points shared by the translation units of libpfgpu.so.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace pf {

struct MultiBufs;   // block-solve buffers (pf_multi.cu)

// Packed-symmetric FP32 storkm (1,830 floats + 2 zero pads per element), by
// cyclic diagonals: D[s][i] = K(i, (i+s) mod 60) at 60 s + i for s = 0..29,
// i = 0..59, and the 30 distinct entries of diagonal 30, K(i, i+30) for
// i = 0..29, at 1800 + i.  Every entry of the symmetric 60 x 60 matrix is
// stored once.  Returns the position of K(i, k), i, k in 0..59.
__host__ __device__ constexpr int packed_off(int i, int k)
{
    const int s = (k - i + 60) % 60;
    return s < 30 ? 60 * s + i : s == 30 ? 1800 + (i < 30 ? i : i - 30) : 60 * (60 - s) + k;
}

// Records a formatted error message for pf_last_error (thread local).
void set_error(const char *fmt, ...);

// The C entry points are function-try-blocks whose handler calls this: a C++
// exception (host memory exhausted, above all) becomes PF_FAILURE with a
// message instead of crossing the C ABI, where it would end the caller.
int host_exception(const char *name);

// Scalars of one PCG run, resident on the device (pinned host mirror).
// Only the single-block finish kernel of an iteration (or block 0 of a
// persistent kernel, after its last barrier of the iteration) writes them,
// so no kernel writes a value that another block of the same kernel reads.
// The one exception is the error path of a grid-wide barrier, which sets
// `stop` so that the run's later launches return at once.
struct PcgState {
    double up;         // r.d entering the next iteration
    double ff;         // f.f (relative-residual denominator)
    double metric;     // last stopping metric
    double rr;         // last r.r
    double alpha;      // batched solves: the iteration's step length, formed once per mesh
    double tol;        // stopping tolerance
    int iters;         // iterations completed
    int stop;          // 1 once converged or at the limit: later kernels return
    int converged;
    int limit;
    int stop_mode;     // 0 checon_par, 1 relative residual
    int err;           // device-detected error code (0 = none)
};

enum { STOP_CHECON = 0, STOP_RELRES = 1 };
constexpr int kPersistSlots = 8;   // persistent-kernel instantiations, one barrier counter and grid each
constexpr int kBarWords = 16;      // u64 words per counter (one 128-byte line each)
// 20-node elasticity (p121), 8-node scalar (p123), 8-node elasticity (p122's demo)
enum { KIND_SOLID20 = 0, KIND_SCALAR8 = 1, KIND_SOLID8 = 2 };

struct Ctx {
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    long long launches = 0;

    int nels = 0, nn = 0, neq = 0, nslots = 0;   // nslots = 3*nn (node-major dofs)
    int *conn = nullptr;        // [nels*20] 0-based node index
    int *node_ptr = nullptr;    // [nn+1] CSR of node -> (element, local node)
    int *node_list = nullptr;   // [nels*20] contribution indices e*20+a, ascending e within a node
    int *slot_eq = nullptr;     // [nslots] 1-based equation or 0 (restrained)
    int *eq_slot = nullptr;     // [neq] slot of equation q+1
    uint8_t *freemask = nullptr;// [nn] bit d set when dof d of the node is free
    double *coord = nullptr;    // [nels*60] g_coord(20,3,e)

    int nmat = 0;               // 1 or nels
    double *mat_e = nullptr, *mat_v = nullptr;

    double *km64 = nullptr;     // [nels*3600] storkm(60,60,e)
    float *km32 = nullptr;      // [nels*3600] full FP32 copy
    float *km32p = nullptr;     // [nels*1832] packed symmetric storkm (packed_off), FP32
    int *kerr = nullptr;        // device error word: 2 = a bulk-copy wait timed out, 3 = a grid barrier did
    bool have_km = false;

    double *ediag = nullptr;    // [nels*60] element diagonals
    double *diag = nullptr;     // [nslots]
    double *dinv = nullptr;     // [nslots] 1/diag, 0 for restrained

    // vectors over slots
    double *f = nullptr, *x = nullptr, *c = nullptr, *r = nullptr, *d = nullptr,
           *p = nullptr, *u = nullptr, *rres = nullptr;
    double *eqbuf = nullptr;    // [neq] staging in equation order
    void *utemp = nullptr;      // element results: FP64 [nels][60], or FP32 [nels][20][4]
                                //   (x, y, z of each local node padded to 16 bytes)
    int stop_mode = 0;          // stopping test of the PCG run in flight
    // CUDA graph of kGraphIters PCG iterations, keyed by what its launches bake in
    cudaGraphExec_t it_graph = nullptr;
    int it_prec = -1, it_stop_mode = -1, it_sym_cfg = -1;
    double *it_xsol = nullptr;
    long long it_launches = 0;  // kernels in one replay
    bool use_graphs = true;
    int kind = 0;               // KIND_SOLID20 (p121), KIND_SCALAR8 (p123) or KIND_SOLID8
    double *fstore = nullptr;   // [nslots] 8-node kinds: penalty store of fixed freedoms, 0 = free
    double *fscale = nullptr;   // [1] KIND_SOLID8: the PCG product at a fixed freedom is p * store * fscale
    // one element matrix shared by every element (PCG_KM); per-element storkm unused
    bool shared = false;
    double *skm64 = nullptr;    // [3600] column-major
    float *skm32 = nullptr;     // [3600 + 192]: km, then the direction sums of its rows ([3][64])
    bool shared_attr = false;   // shared-memory attribute of the tensor-core kernel set
    float2 *psplit = nullptr;   // [nslots] FP32 high and low parts of p (shared km): written with p
    uint32_t *km16p = nullptr;  // [nels*916] packed FP16 storkm (pf_elem_h16.cu), packed on first use
    bool km16_ok = false;       // km16p holds the current storkm
    int h16_cfg = 0;            // autotuned configuration of the FP16 kernel
    unsigned h16_attr = 0;      // FP16 configurations whose shared-memory attribute is set
    float tune16_ms[3] = {0, 0, 0};
    MultiBufs *multi = nullptr; // block-solve vectors, allocated on the first block solve or product
    bool mr_ok = false;         // multi->rec holds the tensor-core element records of the current storkm
    int sym_cfg = 0;            // autotuned configuration of the packed-symmetric kernel
    int sym_warps = 14, sym_stages = 2;
    unsigned long long sym_attr = 0;   // configurations whose shared-memory attribute is set
    float tune_ms[4] = {0, 0, 0, 0};

    // persistent PCG kernels (cooperative launches with grid-wide barriers)
    bool persistent = false;    // true: persistent cooperative kernels for the iteration (pf_set_persistent)
    unsigned long long *gbar = nullptr;   // [kPersistSlots] grid-barrier arrival counters, zeroed per run
    int pk_grid[kPersistSlots] = {};      // blocks of each persistent instantiation (0 = not sized)

    int G = 0;                  // blocks of the vector kernels
    int Gs = 0;                 // blocks of the node scatter
    double *part = nullptr;     // [Gs + 6*G + 16] block partials, split as:
    double *part_s = nullptr;   //   [Gs]  scatter partials (p.u or rres.rres)
    double *part_u = nullptr;   //   [4G]  update partials (r.d, r.r, max|x|, max|dx|)
    double *part_r = nullptr;   //   [2G]  residual-replacement partials
    double *scr = nullptr;      //   [16]  scalars read back by the host
    PcgState *st = nullptr;     // device
    PcgState *hst = nullptr;    // pinned host mirror

    // last solve statistics
    double stats[8] = {0};
};

// Kernel launchers (pf_kernels.cu).  All run on ctx.stream and count launches.
int launch_form_storkm(Ctx &c, int nip, bool exact_weights, bool keep32);
int launch_sample(cudaStream_t stream, int nip, bool exact_weights, double *gp);
int launch_form_storkm_raw(cudaStream_t stream, int nsm, int nels, int nip, const double *gp,
                           const double *coord, const double *me, const double *mv, int nmat, double *km64,
                           float *km32, double *ediag);
int launch_cast_km32(Ctx &c);
int launch_assemble_diag(Ctx &c);
int launch_eq_to_slot(Ctx &c, const double *eq, double *slot);
int launch_slot_to_eq(Ctx &c, const double *slot, double *eq);
// Element products utemp(:,e) = K_e p_e (prec 64 or 32); p is a slot vector.
int launch_elem(Ctx &c, int prec, const double *p);
// Node-centric scatter of utemp: u = sum of contributions (restrained = 0)
// with block partials of p.u (mode 0), or rres = f - sum with partials of
// rres.rres (mode 1).
int launch_scatter(Ctx &c, int prec, int mode, const double *p_or_f, double *out);
int launch_matvec(Ctx &c, int prec, const double *p, double *u);
int launch_residual(Ctx &c, const double *f, const double *x, double *rres);
int launch_scatter_add64(Ctx &c, double *out);   // out += scatter of the FP64 element results in utemp
int launch_pcg_init(Ctx &c, const double *rhs, double *xsol, int stop_mode, double tol, int limit,
                    bool keep_x = false);
int launch_update1(Ctx &c, double *xsol);
int launch_update2(Ctx &c);   // update2 + the one-block finish kernel
int launch_pcg_iteration(Ctx &c, int prec, double *xsol);
// Persistent forms: the scatter + updates + finish of one iteration in one
// cooperative launch (after the element products), and whole FP64
// iterations (element products included), up to niters per launch.
int launch_pcg_tail(Ctx &c, int prec, double *xsol);
int launch_pcg_fused64(Ctx &c, double *xsol, int niters);
bool persist_fused64(const Ctx &c, int prec);
// One bounded mbarrier wait that nothing completes (the error path of the
// bulk-copy kernels, without a fault): records code 2 in c.kerr.
int launch_wait_probe(Ctx &c, long long polls);
int launch_axpy(Ctx &c, double *y, const double *xv);          // y += x
int launch_replace(Ctx &c, double tol);   // r = rres, d = diag*r, up = r.d; p kept
int launch_sum_partials(Ctx &c, int nvals, double *out_dev);   // out[0] = sum of part_s
int launch_centroid_stress(Ctx &c, int e0, int count, const double *xslot, double *sig_dev);
// prec codes of the element products: 64 FP64 storkm, 32 packed-symmetric
// FP32 storkm (bulk-copy staged), 31 full FP32 storkm
enum { PREC_FP64 = 64, PREC_FP32_SYM = 32, PREC_FP32_FULL = 31, PREC_FP16_SYM = 16 };
int ensure_km16(Ctx &c);   // packs (and autotunes) the FP16 storkm if storkm changed; outside stream capture
int launch_elem_sym16(Ctx &c, const double *p, const PcgState *st);
int h16_config(int idx, int *warps, int *stages);
int sym16_prepare();   // shared-memory attribute of the mapped FP16 launch (once per device, outside capture)
int launch_elem_sym16_mapped(cudaStream_t stream, int nsm, int n, const uint32_t *kh, const int *conn,
                             const double *p, float *ut, int *err, const int *emap);
int launch_pack_sym16_raw(cudaStream_t stream, int nsm, int nels, const double *km, uint32_t *kh);
int launch_pack_sym32(Ctx &c);
void multi_release(Ctx &c);   // frees the context's block-solve buffers (pf_multi.cu)
int launch_elem_sym32(Ctx &c, const double *p, const PcgState *st);
int sym32_prepare();   // shared-memory attribute of the mapped launch (once per device, outside capture)
int launch_elem_sym32_mapped(cudaStream_t stream, int nsm, int n, const float *kp, const int *conn, const double *p,
                             float *ut, int *err, const int *emap);
int launch_pack_sym32_raw(cudaStream_t stream, int nsm, int nels, const double *km, float *kp);
int autotune_sym32(Ctx &c, const double *p);   // picks c.sym_cfg by timing on this mesh
int launch_elem_shared(Ctx &c, int prec, const double *p, const PcgState *st);   // shared km
// 8-node scalar (p123) kernels; km64 holds storkc(8,8,e) in such a context
int launch_form_storkc(Ctx &c, int nip, double kx, double ky, double kz);
int launch_elem8(Ctx &c, const double *p, const PcgState *st);
int launch_scatter1(Ctx &c, int mode, const double *xin, const double *pf, double *out, const PcgState *st);
int launch_assemble_diag1(Ctx &c);
int launch_set_fixed(Ctx &c, int nfix, const int *slots_dev, double penalty);
// pf_solid8.cu: 8-node elasticity bricks (24 freedoms per element), FP64
int launch_elem24(Ctx &c, const double *p, const PcgState *st);
int launch_scatter3_fixed(Ctx &c, const double *p, double *out, const PcgState *st);
int launch_shared_ediag(Ctx &c);
void set_sym_config(Ctx &c, int idx);           // 0: 14 warps x 2 stages, 1: 12 x 2, 2: 8 x 3
int launch_matvec_generic(int n_mat, int n_row, int n_col, const double *lhs,
                          const double *mat, double *rhs, long long *launches);

}  // namespace pf
