// pf_abi.cu -- the C-ABI of libpfgpu.so (declared in include/pfgpu.h).
//
// Host side of the solve layer: context lifetime, mesh set-up (the
// node-centric scatter tables that replace MAKE_GGL's halo tables,
// src/modules/mpi/gather_scatter.f90:1387-1784), and the solve drivers of
// p121.f90:86-104.  All device work is issued on the context's stream; every
// entry point synchronises before it returns, as xx3's layer does
// (src/programs/dev/xx3/cuda_helpers.cu:355-365).
#include "pf_internal.h"
#include "pfgpu.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

namespace pf {

static thread_local std::string g_err;

void set_error(const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
}

int host_exception(const char *name)
{
    try {
        throw;
    } catch (const std::bad_alloc &) {
        set_error("%s: out of host memory", name);
    } catch (const std::exception &e) {
        set_error("%s: %s", name, e.what());
    } catch (...) {
        set_error("%s: unexpected C++ exception", name);
    }
    return PF_FAILURE;
}

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return PF_FAILURE;                                                           \
        }                                                                                \
    } while (0)

#define TRY(call)                        \
    do {                                 \
        if ((call) != 0) return PF_FAILURE; \
    } while (0)

template <typename T>
static int dalloc(T **ptr, size_t count, const char *what)
{
    *ptr = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)ptr, count * sizeof(T));
    if (e != cudaSuccess) {
        set_error("cannot allocate %s (%zu bytes): %s", what, count * sizeof(T), cudaGetErrorString(e));
        *ptr = nullptr;
        return 1;
    }
    return 0;
}

template <typename T>
static void dfree(T *&p)
{
    if (p) cudaFree((void *)p);
    p = nullptr;
}

static Ctx *get_ctx(void **h)
{
    if (!h || !*h) {
        set_error("null solver context");
        return nullptr;
    }
    Ctx *c = (Ctx *)*h;
    if (cudaSetDevice(c->device) != cudaSuccess) {
        set_error("cannot select device %d", c->device);
        return nullptr;
    }
    return c;
}

static void drop_graph(Ctx &c)
{
    if (c.it_graph) cudaGraphExecDestroy(c.it_graph);
    c.it_graph = nullptr;
    c.it_prec = c.it_stop_mode = c.it_sym_cfg = -1;
    c.it_xsol = nullptr;
    c.it_launches = 0;
}

static void free_mesh(Ctx &c)
{
    drop_graph(c);
    multi_release(c);
    dfree(c.conn); dfree(c.node_ptr); dfree(c.node_list); dfree(c.slot_eq); dfree(c.eq_slot);
    dfree(c.freemask); dfree(c.coord); dfree(c.mat_e); dfree(c.mat_v); dfree(c.km64); dfree(c.km32);
    dfree(c.km32p); dfree(c.skm64); dfree(c.skm32); dfree(c.fstore); dfree(c.fscale); dfree(c.psplit);
    dfree(c.km16p);
    c.km16_ok = false;
    c.mr_ok = false;
    c.shared = false;
    c.kind = KIND_SOLID20;
    dfree(c.ediag); dfree(c.diag); dfree(c.dinv); dfree(c.f); dfree(c.x); dfree(c.c); dfree(c.r);
    dfree(c.d); dfree(c.p); dfree(c.u); dfree(c.rres); dfree(c.eqbuf); dfree(c.utemp); dfree(c.part);
    c.nels = c.nn = c.neq = c.nslots = 0;
    c.nmat = 0;
    c.have_km = false;
    for (int &g : c.pk_grid) g = 0;
}

static int sync(Ctx &c)
{
    CK(cudaStreamSynchronize(c.stream));
    return 0;
}

// Reads the device PCG state into the pinned mirror.
static int pull_state(Ctx &c)
{
    CK(cudaMemcpyAsync(c.hst, c.st, sizeof(PcgState), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return 0;
}

// Reads and clears the bulk-copy kernels' device error word.
static int check_kernel_error(Ctx &c)
{
    int err = 0;
    CK(cudaMemcpyAsync(&err, c.kerr, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (err) {
        cudaMemsetAsync(c.kerr, 0, sizeof(int), c.stream);
        cudaStreamSynchronize(c.stream);
        if (err == 3)
            set_error("persistent PCG kernel: a grid-wide barrier wait timed out (code 3)");
        else
            set_error("element kernel: a shared-memory bulk-copy wait timed out (code %d)", err);
        return 1;
    }
    return 0;
}

constexpr int kGraphIters = 8;   // PCG iterations per graph replay

// The graph of kGraphIters iterations for (prec, xsol) under the current
// stopping test and element-kernel configuration, captured on first use.
static int iteration_graph(Ctx &c, int prec, double *xsol, cudaGraphExec_t *out)
{
    if (c.it_graph && c.it_prec == prec && c.it_xsol == xsol && c.it_stop_mode == c.stop_mode &&
        c.it_sym_cfg == c.sym_cfg) {
        *out = c.it_graph;
        return 0;
    }
    drop_graph(c);
    const long long l0 = c.launches;
    CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    int bad = 0;
    for (int i = 0; i < kGraphIters && !bad; ++i) bad = launch_pcg_iteration(c, prec, xsol);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(c.stream, &g);
    if (bad || ec != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        if (!bad) set_error("PCG iteration graph: capture failed: %s", cudaGetErrorString(ec));
        c.launches = l0;
        return 1;
    }
    const cudaError_t ei = cudaGraphInstantiate(&c.it_graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        c.it_graph = nullptr;
        set_error("PCG iteration graph: instantiate failed: %s", cudaGetErrorString(ei));
        c.launches = l0;
        return 1;
    }
    c.it_launches = c.launches - l0;
    c.launches = l0;
    c.it_prec = prec;
    c.it_xsol = xsol;
    c.it_stop_mode = c.stop_mode;
    c.it_sym_cfg = c.sym_cfg;
    *out = c.it_graph;
    return 0;
}

// Runs PCG iterations until the device state says stop.  The state is read
// back every `chunk` iterations; iterations launched after the stop return
// at once (every kernel checks the flag).  Whole groups of kGraphIters
// iterations are replayed from a CUDA graph (one launch instead of five
// per iteration); the remainder below the limit is launched directly.
static int run_pcg(Ctx &c, int prec, double *xsol, int limit)
{
    int launched = 0;
    int chunk = 4;
    if (persist_fused64(c, prec)) {
        // whole FP64 iterations in persistent launches, one launch per chunk
        for (;;) {
            const int todo = chunk < limit - launched ? chunk : limit - launched;
            if (todo > 0) TRY(launch_pcg_fused64(c, xsol, todo));
            launched += todo;
            TRY(pull_state(c));
            if (c.hst->stop || launched >= limit) break;
            if (chunk < 32) chunk *= 2;
        }
        if (check_kernel_error(c)) return 1;
        if (c.hst->err) {
            set_error("PCG breakdown after %d iterations (non-finite r.d or |x|)", c.hst->iters);
            return 1;
        }
        return 0;
    }
    for (;;) {
        int todo = chunk < limit - launched ? chunk : limit - launched;
        if (c.use_graphs && todo >= kGraphIters) {
            cudaGraphExec_t ge = nullptr;
            TRY(iteration_graph(c, prec, xsol, &ge));
            for (; todo >= kGraphIters; todo -= kGraphIters, launched += kGraphIters) {
                CK(cudaGraphLaunch(ge, c.stream));
                c.launches += c.it_launches;
            }
        }
        for (; todo > 0; --todo, ++launched) TRY(launch_pcg_iteration(c, prec, xsol));
        TRY(pull_state(c));
        if (c.hst->stop || launched >= limit) break;
        if (chunk < 32) chunk *= 2;
    }
    if (check_kernel_error(c)) return 1;
    if (c.hst->err) {
        set_error("PCG breakdown after %d iterations (non-finite r.d or |x|)", c.hst->iters);
        return 1;
    }
    return 0;
}

int run_pcg_public(Ctx &c, int prec, double *xsol, int limit) { return run_pcg(c, prec, xsol, limit); }

// ||f - K64 x||_2 / ||f||_2 on the device (fills c.rres).
static int true_relres(Ctx &c, const double *x, double ff, double *out, double *dev2)
{
    TRY(launch_residual(c, c.f, x, c.rres));
    TRY(launch_sum_partials(c, 1, dev2));
    double rr = 0.0;
    CK(cudaMemcpyAsync(&rr, dev2, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    *out = ff > 0.0 ? std::sqrt(rr) / std::sqrt(ff) : 0.0;
    return 0;
}

}  // namespace pf

using namespace pf;

// ===========================================================================
// xx3 layer (src/programs/dev/xx3/cuda_helpers.cu:183-368)
extern "C" int set_gpu(const int *device_id)
try {
    if (!device_id) { set_error("set_gpu: null argument"); return PF_FAILURE; }
    CK(cudaSetDevice(*device_id));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("set_gpu");
}

extern "C" int allocate_memory_on_gpu(const int *n_elements, const int *element_size, void **device_pointer)
try {
    if (!n_elements || !element_size || !device_pointer || *n_elements < 0 || *element_size < 0) {
        set_error("allocate_memory_on_gpu: invalid arguments");
        return PF_FAILURE;
    }
    const size_t bytes = (size_t)*n_elements * (size_t)*element_size;
    CK(cudaMalloc(device_pointer, bytes ? bytes : 1));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("allocate_memory_on_gpu");
}

extern "C" int free_memory_on_gpu(void **device_pointer)
try {
    if (!device_pointer) { set_error("free_memory_on_gpu: null argument"); return PF_FAILURE; }
    CK(cudaFree(*device_pointer));
    *device_pointer = nullptr;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("free_memory_on_gpu");
}

extern "C" int copy_data_to_gpu(const int *n_elements, const int *element_size, const void *host_data,
                                void **device_pointer)
try {
    if (!n_elements || !element_size || !device_pointer || (!host_data && *n_elements > 0)) {
        set_error("copy_data_to_gpu: invalid arguments");
        return PF_FAILURE;
    }
    CK(cudaMemcpy(*device_pointer, host_data, (size_t)*n_elements * (size_t)*element_size,
                  cudaMemcpyHostToDevice));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("copy_data_to_gpu");
}

extern "C" int copy_data_from_gpu(const int *n_elements, const int *element_size, void *host_data,
                                  void **device_pointer)
try {
    if (!n_elements || !element_size || !device_pointer || (!host_data && *n_elements > 0)) {
        set_error("copy_data_from_gpu: invalid arguments");
        return PF_FAILURE;
    }
    CK(cudaMemcpy(host_data, *device_pointer, (size_t)*n_elements * (size_t)*element_size,
                  cudaMemcpyDeviceToHost));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("copy_data_from_gpu");
}

static long long g_xx3_launches = 0;

extern "C" int matrix_vector_multiplies(int *n_mat, int *n_row, int *n_col, void **d_lhs_vector,
                                        void **d_matrix, void **d_rhs_vector)
try {
    if (!n_mat || !n_row || !n_col || !d_lhs_vector || !d_matrix || !d_rhs_vector || *n_mat < 0 ||
        *n_row < 1 || *n_col < 1) {
        set_error("matrix_vector_multiplies: invalid arguments");
        return PF_FAILURE;
    }
    if (*n_mat == 0) return PF_SUCCESS;
    if (launch_matvec_generic(*n_mat, *n_row, *n_col, (const double *)*d_lhs_vector,
                              (const double *)*d_matrix, (double *)*d_rhs_vector, &g_xx3_launches))
        return PF_FAILURE;
    CK(cudaDeviceSynchronize());
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("matrix_vector_multiplies");
}

// ===========================================================================
// solve layer
extern "C" int pf_last_error(char *buf, const int *len)
try {
    if (!buf || !len || *len <= 0) return PF_FAILURE;
    const size_t n = (size_t)*len - 1;
    const size_t m = g_err.size() < n ? g_err.size() : n;
    memcpy(buf, g_err.data(), m);
    buf[m] = '\0';
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_last_error");
}

extern "C" int pf_ctx_create(const int *device, void **ctx)
try {
    if (!device || !ctx) { set_error("pf_ctx_create: null argument"); return PF_FAILURE; }
    *ctx = nullptr;
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (*device < 0 || *device >= ndev) {
        set_error("pf_ctx_create: device %d out of range (%d devices)", *device, ndev);
        return PF_FAILURE;
    }
    CK(cudaSetDevice(*device));
    Ctx *c = new (std::nothrow) Ctx();
    if (!c) { set_error("pf_ctx_create: out of host memory"); return PF_FAILURE; }
    c->device = *device;
    cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device);
    if (c->nsm < 1) c->nsm = 1;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc((void **)&c->st, sizeof(PcgState)) != cudaSuccess ||
        cudaMalloc((void **)&c->kerr, sizeof(int)) != cudaSuccess ||
        cudaMemset(c->kerr, 0, sizeof(int)) != cudaSuccess ||
        cudaMalloc((void **)&c->gbar, sizeof(unsigned long long) * kPersistSlots * kBarWords) != cudaSuccess ||
        cudaMemset(c->gbar, 0, sizeof(unsigned long long) * kPersistSlots * kBarWords) != cudaSuccess ||
        cudaMallocHost((void **)&c->hst, sizeof(PcgState)) != cudaSuccess) {
        set_error("pf_ctx_create: cannot create stream/state");
        if (c->stream) cudaStreamDestroy(c->stream);
        if (c->st) cudaFree(c->st);
        delete c;
        return PF_FAILURE;
    }
    memset(c->hst, 0, sizeof(PcgState));
    *ctx = c;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_ctx_create");
}

extern "C" int pf_ctx_destroy(void **ctx)
try {
    if (!ctx || !*ctx) return PF_SUCCESS;
    Ctx *c = (Ctx *)*ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_mesh(*c);   // also drops the iteration graph
    if (c->st) cudaFree(c->st);
    if (c->kerr) cudaFree(c->kerr);
    if (c->gbar) cudaFree(c->gbar);
    if (c->hst) cudaFreeHost(c->hst);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    *ctx = nullptr;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_ctx_destroy");
}

// Mesh tables of a context: nod nodes per element (20 or 8) with nodof
// freedoms per node (3 or 1).  Slots are node-major (nodof * node + dof).
static int setup_mesh(void **ctx, const int *nels_p, const int *nn_p, const int *neq_p, const int *g_num,
                      const int *g_g, const double *g_coord, const int nod, const int nodof)
{
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (!nels_p || !nn_p || !neq_p || !g_num || !g_g || !g_coord) {
        set_error("pf_setup: null argument");
        return PF_FAILURE;
    }
    const int ntot = nod * nodof;
    const int nels = *nels_p, nn = *nn_p, neq = *neq_p;
    if (nels < 1 || nn < 1 || neq < 0 || (long long)nn * nodof > 0x7fffffffLL ||
        (long long)nels * 60 > 0x7fffffffLL) {
        set_error("pf_setup: invalid sizes nels=%d nn=%d neq=%d", nels, nn, neq);
        return PF_FAILURE;
    }
    CK(cudaStreamSynchronize(c.stream));
    free_mesh(c);
    const int ns = nodof * nn;
    std::vector<int> conn((size_t)nels * nod), slot_eq(ns, -1), eq_slot(neq > 0 ? neq : 1, -1);
    std::vector<int> cnt(nn + 1, 0);
    for (size_t e = 0; e < (size_t)nels; ++e)
        for (int a = 0; a < nod; ++a) {
            const int nd = g_num[e * nod + a];
            if (nd < 1 || nd > nn) {
                set_error("pf_setup: g_num(%d,%zu)=%d outside 1..%d", a + 1, e + 1, nd, nn);
                return PF_FAILURE;
            }
            conn[e * nod + a] = nd - 1;
            cnt[nd]++;
            for (int d = 0; d < nodof; ++d) {
                const int q = g_g[e * ntot + nodof * a + d];
                if (q < 0 || q > neq) {
                    set_error("pf_setup: g_g(%d,%zu)=%d outside 0..%d", nodof * a + d + 1, e + 1, q, neq);
                    return PF_FAILURE;
                }
                int &se = slot_eq[nodof * (nd - 1) + d];
                if (se < 0) se = q;
                else if (se != q) {
                    set_error("pf_setup: node %d dof %d has equations %d and %d in different elements", nd,
                              d + 1, se, q);
                    return PF_FAILURE;
                }
            }
        }
    std::vector<uint8_t> fm(nn, 0);
    for (int s = 0; s < ns; ++s) {
        if (slot_eq[s] < 0) slot_eq[s] = 0;   // node used by no element
        const int q = slot_eq[s];
        if (q > 0) {
            if (eq_slot[q - 1] >= 0) {
                set_error("pf_setup: equation %d belongs to two dofs", q);
                return PF_FAILURE;
            }
            eq_slot[q - 1] = s;
            fm[s / nodof] |= (uint8_t)(1u << (s % nodof));
        }
    }
    for (int q = 0; q < neq; ++q)
        if (eq_slot[q] < 0) {
            set_error("pf_setup: equation %d is not used by any element", q + 1);
            return PF_FAILURE;
        }
    // node -> (element, local node) table, ascending element order per node
    std::vector<int> ptr(nn + 1, 0);
    for (int n = 0; n < nn; ++n) ptr[n + 1] = ptr[n] + cnt[n + 1];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1), list((size_t)nels * nod);
    for (size_t e = 0; e < (size_t)nels; ++e)
        for (int a = 0; a < nod; ++a) {
            const int n = conn[e * nod + a];
            list[fill[n]++] = (int)(e * nod + a);   // contribution index: element e, local node a
        }

    c.nels = nels; c.nn = nn; c.neq = neq; c.nslots = ns;
    c.kind = nod == 8 ? (nodof == 1 ? KIND_SCALAR8 : KIND_SOLID8) : KIND_SOLID20;
    long long g = ((long long)ns + 255) / 256;
    if (g > (long long)c.nsm * 8) g = (long long)c.nsm * 8;
    c.G = (int)(g < 1 ? 1 : g);
    long long gs = ((long long)nn + 255) / 256;
    if (gs > (long long)c.nsm * 16) gs = (long long)c.nsm * 16;
    c.Gs = (int)(gs < 1 ? 1 : gs);
    const size_t ne = (size_t)nels;
    if (dalloc(&c.conn, ne * nod, "connectivity") || dalloc(&c.node_ptr, nn + 1, "node table") ||
        dalloc(&c.node_list, ne * nod, "node table") || dalloc(&c.slot_eq, ns, "slot map") ||
        dalloc(&c.eq_slot, neq, "equation map") || dalloc(&c.freemask, nn, "restraint mask") ||
        dalloc(&c.coord, ne * nod * 3, "coordinates") || dalloc(&c.ediag, ne * ntot, "element diagonals") ||
        (nod == 8 && dalloc(&c.fstore, ns, "fixed freedoms")) ||
        (c.kind == KIND_SOLID8 && dalloc(&c.fscale, 1, "fixed-freedom factor")) ||
        dalloc(&c.diag, ns, "diag") || dalloc(&c.dinv, ns, "diag") || dalloc(&c.f, ns, "f") ||
        dalloc(&c.x, ns, "x") || dalloc(&c.c, ns, "c") || dalloc(&c.r, ns, "r") || dalloc(&c.d, ns, "d") ||
        dalloc(&c.p, ns, "p") || dalloc(&c.u, ns, "u") || dalloc(&c.rres, ns, "rres") ||
        dalloc(&c.eqbuf, neq + 8, "equation buffer") || dalloc((double **)&c.utemp, ne * ntot, "utemp") ||
        dalloc(&c.part, (size_t)c.Gs + 6 * (size_t)c.G + 16, "partials")) {
        free_mesh(c);
        return PF_FAILURE;
    }
    c.part_s = c.part;
    c.part_u = c.part_s + c.Gs;
    c.part_r = c.part_u + 4 * (size_t)c.G;
    c.scr = c.part_r + 2 * (size_t)c.G;
    CK(cudaMemcpyAsync(c.conn, conn.data(), ne * nod * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.node_ptr, ptr.data(), (nn + 1) * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.node_list, list.data(), ne * nod * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.slot_eq, slot_eq.data(), ns * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    if (neq > 0)
        CK(cudaMemcpyAsync(c.eq_slot, eq_slot.data(), neq * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.freemask, fm.data(), nn, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.coord, g_coord, ne * nod * 3 * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    if (c.fstore) CK(cudaMemsetAsync(c.fstore, 0, ns * sizeof(double), c.stream));
    if (c.fscale) {
        static const double one = 1.0;
        CK(cudaMemcpyAsync(c.fscale, &one, sizeof(double), cudaMemcpyHostToDevice, c.stream));
    }
    CK(cudaMemsetAsync(c.x, 0, ns * sizeof(double), c.stream));
    CK(cudaMemsetAsync(c.f, 0, ns * sizeof(double), c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return PF_SUCCESS;
}

extern "C" int pf_setup(void **ctx, const int *nels, const int *nn, const int *neq, const int *g_num,
                        const int *g_g, const double *g_coord)
try {
    return setup_mesh(ctx, nels, nn, neq, g_num, g_g, g_coord, 20, 3);
} catch (...) {
    return pf::host_exception("pf_setup");
}

extern "C" int pf_setup_scalar8(void **ctx, const int *nels, const int *nn, const int *neq, const int *g_num,
                                const int *g_g, const double *g_coord)
try {
    return setup_mesh(ctx, nels, nn, neq, g_num, g_g, g_coord, 8, 1);
} catch (...) {
    return pf::host_exception("pf_setup_scalar8");
}

extern "C" int pf_setup_solid8(void **ctx, const int *nels, const int *nn, const int *neq, const int *g_num,
                               const int *g_g, const double *g_coord)
try {
    return setup_mesh(ctx, nels, nn, neq, g_num, g_g, g_coord, 8, 3);
} catch (...) {
    return pf::host_exception("pf_setup_solid8");
}

extern "C" int pf_form_storkc(void **ctx, const int *nip, const double *kx, const double *ky, const double *kz)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (c.kind != KIND_SCALAR8 || c.nels == 0) {
        set_error("pf_form_storkc: call pf_setup_scalar8 first");
        return PF_FAILURE;
    }
    if (!nip || !kx || !ky || !kz || (*nip != 8 && *nip != 27)) {
        set_error("pf_form_storkc: nip must be 8 or 27");
        return PF_FAILURE;
    }
    if (!c.km64 && dalloc(&c.km64, (size_t)c.nels * 64, "storkc")) return PF_FAILURE;
    drop_graph(c);
    TRY(launch_form_storkc(c, *nip, *kx, *ky, *kz));
    TRY(launch_assemble_diag(c));
    TRY(sync(c));
    c.have_km = true;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_form_storkc");
}

extern "C" int pf_get_storkc(void **ctx, const int *first, const int *count, double *storkc)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (c.kind != KIND_SCALAR8 || !c.have_km || !first || !count || !storkc || *first < 0 || *count < 0 ||
        *first + (long long)*count > c.nels) {
        set_error("pf_get_storkc: invalid range or no storkc");
        return PF_FAILURE;
    }
    CK(cudaMemcpyAsync(storkc, c.km64 + (size_t)*first * 64, (size_t)*count * 64 * sizeof(double),
                       cudaMemcpyDeviceToHost, c.stream));
    TRY(sync(c));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_get_storkc");
}

extern "C" int pf_set_fixed(void **ctx, const int *nfix, const int *eqs, const double *penalty)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if ((c.kind != KIND_SCALAR8 && c.kind != KIND_SOLID8) || !c.have_km) {
        set_error("pf_set_fixed: needs an 8-node context with its element matrices formed");
        return PF_FAILURE;
    }
    if (!nfix || *nfix < 0 || (*nfix > 0 && !eqs) || !penalty) {
        set_error("pf_set_fixed: invalid arguments");
        return PF_FAILURE;
    }
    if (*nfix == 0) return PF_SUCCESS;
    std::vector<int> slot_eq(c.nslots), slots(*nfix);
    CK(cudaMemcpy(slot_eq.data(), c.slot_eq, (size_t)c.nslots * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<int> eq_slot(c.neq + 1, -1);
    for (int s = 0; s < c.nslots; ++s)
        if (slot_eq[s] > 0) eq_slot[slot_eq[s]] = s;
    for (int i = 0; i < *nfix; ++i) {
        if (eqs[i] < 1 || eqs[i] > c.neq) {
            set_error("pf_set_fixed: equation %d outside 1..%d", eqs[i], c.neq);
            return PF_FAILURE;
        }
        slots[i] = eq_slot[eqs[i]];
    }
    int *d_slots = nullptr;
    if (dalloc(&d_slots, (size_t)*nfix, "fixed freedoms")) return PF_FAILURE;
    cudaError_t e = cudaMemcpyAsync(d_slots, slots.data(), (size_t)*nfix * sizeof(int), cudaMemcpyHostToDevice,
                                    c.stream);
    int bad = e != cudaSuccess;
    if (!bad) bad = launch_set_fixed(c, *nfix, d_slots, *penalty);
    if (!bad) bad = sync(c);
    cudaFree(d_slots);
    if (bad && e != cudaSuccess) set_error("pf_set_fixed: %s", cudaGetErrorString(e));
    drop_graph(c);
    return bad ? PF_FAILURE : PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_set_fixed");
}

extern "C" int pf_set_material(void **ctx, const int *n, const double *e, const double *v)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (!n || !e || !v || c.nels == 0 || (*n != 1 && *n != c.nels)) {
        set_error("pf_set_material: n must be 1 or nels (after pf_setup)");
        return PF_FAILURE;
    }
    for (int i = 0; i < *n; ++i)
        if (!(e[i] > 0.0) || !(v[i] > -1.0 && v[i] < 0.5)) {
            set_error("pf_set_material: invalid E=%g v=%g for element %d", e[i], v[i], i + 1);
            return PF_FAILURE;
        }
    dfree(c.mat_e);
    dfree(c.mat_v);
    if (dalloc(&c.mat_e, *n, "material") || dalloc(&c.mat_v, *n, "material")) return PF_FAILURE;
    c.nmat = *n;
    CK(cudaMemcpyAsync(c.mat_e, e, *n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.mat_v, v, *n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_set_material");
}

// The per-element storkm arrays (FP64, FP32, packed FP32), allocated on the
// first pf_form_storkm / pf_set_storkm: a context that only ever uses a
// shared element matrix never holds them.
static int ensure_storkm(Ctx &c)
{
    const size_t ne = (size_t)c.nels;
    if (c.kind == KIND_SOLID8) {   // FP64 storkm(24,24,e) only
        if (!c.km64 && dalloc(&c.km64, ne * 576, "FP64 storkm")) return 1;
        drop_graph(c);
        return 0;
    }
    if (!c.km64 && dalloc(&c.km64, ne * 3600, "FP64 storkm")) return 1;
    if (!c.km32 && dalloc(&c.km32, ne * 3600, "FP32 storkm")) return 1;
    if (!c.km32p && dalloc(&c.km32p, ne * 1832, "packed FP32 storkm")) return 1;
    c.km16_ok = false;   // repacked on the next FP16 use
    c.mr_ok = false;     // and the tensor-core block records on the next block product
    c.shared = false;
    drop_graph(c);
    return 0;
}

extern "C" int pf_form_storkm(void **ctx, const int *nip, const int *flags)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (c.kind != KIND_SOLID20 && c.kind != KIND_SOLID8) {
        set_error("pf_form_storkm: needs an elasticity context (pf_setup or pf_setup_solid8)");
        return PF_FAILURE;
    }
    if (!nip || !flags || (*nip != 8 && *nip != 27)) {
        set_error("pf_form_storkm: nip must be 8 or 27");
        return PF_FAILURE;
    }
    if (c.nels == 0 || c.nmat == 0) {
        set_error("pf_form_storkm: call pf_setup and pf_set_material first");
        return PF_FAILURE;
    }
    const bool exact = (*flags & PF_FORM_EXACT_WEIGHTS) != 0;
    TRY(ensure_storkm(c));
    if (c.kind == KIND_SOLID8) {   // FP64 storkm, the diagonal; fixed freedoms cleared
        TRY(launch_form_storkm(c, *nip, exact, false));
        TRY(launch_assemble_diag(c));
        CK(cudaMemsetAsync(c.fstore, 0, (size_t)c.nslots * sizeof(double), c.stream));
        TRY(sync(c));
        c.have_km = true;
        return PF_SUCCESS;
    }
    TRY(launch_form_storkm(c, *nip, exact, true));
    TRY(launch_pack_sym32(c));
    TRY(launch_assemble_diag(c));
    TRY(autotune_sym32(c, c.x));
    TRY(sync(c));
    c.have_km = true;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_form_storkm");
}

extern "C" int pf_set_storkm(void **ctx, const double *storkm)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (c.kind != KIND_SOLID20) {
        set_error("pf_set_storkm: needs a 20-node context (pf_setup)");
        return PF_FAILURE;
    }
    if (!storkm || c.nels == 0) { set_error("pf_set_storkm: call pf_setup first"); return PF_FAILURE; }
    TRY(ensure_storkm(c));
    CK(cudaMemcpyAsync(c.km64, storkm, (size_t)c.nels * 3600 * sizeof(double), cudaMemcpyHostToDevice,
                       c.stream));
    TRY(launch_cast_km32(c));
    TRY(launch_pack_sym32(c));
    TRY(launch_assemble_diag(c));
    TRY(autotune_sym32(c, c.x));
    TRY(sync(c));
    c.have_km = true;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_set_storkm");
}

extern "C" int pf_form_km(void **ctx, const int *iel, const int *nip, const int *flags, double *km)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (c.kind != KIND_SOLID20) {
        set_error("pf_form_km: needs a 20-node context (pf_setup)");
        return PF_FAILURE;
    }
    if (!iel || !nip || !flags || !km || (*nip != 8 && *nip != 27)) {
        set_error("pf_form_km: nip must be 8 or 27");
        return PF_FAILURE;
    }
    if (c.nels == 0 || c.nmat == 0 || *iel < 1 || *iel > c.nels) {
        set_error("pf_form_km: element %d is not in the mesh, or no material", iel ? *iel : 0);
        return PF_FAILURE;
    }
    const size_t e = (size_t)*iel - 1;
    double *buf = nullptr;   // Gauss table (108) + km (3600) + element diagonal (60)
    if (dalloc(&buf, 108 + 3600 + 60, "element matrix")) return PF_FAILURE;
    const int m = c.nmat == 1 ? 0 : (int)e;
    int bad = launch_sample(c.stream, *nip, (*flags & PF_FORM_EXACT_WEIGHTS) != 0, buf);
    if (!bad)
        bad = launch_form_storkm_raw(c.stream, c.nsm, 1, *nip, buf, c.coord + e * 60, c.mat_e + m, c.mat_v + m, 1,
                                     buf + 108, nullptr, buf + 108 + 3600);
    if (!bad) c.launches += 2;
    cudaError_t ec = bad ? cudaSuccess : cudaMemcpyAsync(km, buf + 108, 3600 * sizeof(double), cudaMemcpyDeviceToHost,
                                                         c.stream);
    if (ec == cudaSuccess) ec = cudaStreamSynchronize(c.stream);
    cudaFree(buf);
    if (bad) return PF_FAILURE;
    if (ec != cudaSuccess) {
        set_error("pf_form_km: %s", cudaGetErrorString(ec));
        return PF_FAILURE;
    }
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_form_km");
}

extern "C" int pf_set_shared_km(void **ctx, const double *km)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (c.kind != KIND_SOLID20) {
        set_error("pf_set_shared_km: needs a 20-node context (pf_setup)");
        return PF_FAILURE;
    }
    if (!km || c.nels == 0) {
        set_error("pf_set_shared_km: call pf_setup first");
        return PF_FAILURE;
    }
    for (int i = 0; i < 60; ++i)
        if (!(km[61 * i] > 0.0) || !std::isfinite(km[61 * i])) {
            set_error("pf_set_shared_km: km(%d,%d) = %g is not a positive stiffness", i + 1, i + 1, km[61 * i]);
            return PF_FAILURE;
        }
    if (!c.skm64 && dalloc(&c.skm64, 3600, "shared km")) return PF_FAILURE;
    if (!c.skm32 && dalloc(&c.skm32, 3600 + 192, "shared km")) return PF_FAILURE;
    if (!c.psplit && dalloc(&c.psplit, (size_t)c.nslots, "split search direction")) return PF_FAILURE;
    // FP32 km, then the direction sums of its rows, sum over a of K(3a + d, k)
    // at 3600 + 64d + k (summed in FP64, zero for k = 60..63): the tensor-core
    // product's A operand carries them to remove the results' mean translation
    std::vector<float> k32(3600 + 192, 0.0f);
    for (int i = 0; i < 3600; ++i) k32[i] = (float)km[i];
    for (int d = 0; d < 3; ++d)
        for (int k = 0; k < 60; ++k) {
            double sum = 0.0;
            for (int a = 0; a < 20; ++a) sum += (double)k32[3 * a + d + 60 * k];
            k32[3600 + 64 * d + k] = (float)sum;
        }
    CK(cudaMemcpyAsync(c.skm64, km, 3600 * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.skm32, k32.data(), (3600 + 192) * sizeof(float), cudaMemcpyHostToDevice, c.stream));
    c.shared = true;
    drop_graph(c);
    TRY(launch_shared_ediag(c));
    TRY(launch_assemble_diag(c));
    TRY(sync(c));
    c.have_km = true;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_set_shared_km");
}

extern "C" int pf_get_storkm(void **ctx, const int *first, const int *count, double *storkm)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (c.kind != KIND_SOLID20 && c.kind != KIND_SOLID8) {
        set_error("pf_get_storkm: needs an elasticity context (pf_setup or pf_setup_solid8)");
        return PF_FAILURE;
    }
    if (c.shared) {
        set_error("pf_get_storkm: the context uses one shared element matrix (pf_set_shared_km)");
        return PF_FAILURE;
    }
    if (!first || !count || !storkm || !c.have_km || *first < 0 || *count < 0 || *first + *count > c.nels) {
        set_error("pf_get_storkm: invalid range or no storkm");
        return PF_FAILURE;
    }
    const size_t ke = c.kind == KIND_SOLID8 ? 576 : 3600;
    CK(cudaMemcpyAsync(storkm, c.km64 + (size_t)*first * ke, (size_t)*count * ke * sizeof(double),
                       cudaMemcpyDeviceToHost, c.stream));
    TRY(sync(c));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_get_storkm");
}

extern "C" int pf_get_diag(void **ctx, double *diag)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (!diag || !c.have_km) { set_error("pf_get_diag: no storkm"); return PF_FAILURE; }
    TRY(launch_slot_to_eq(c, c.diag, c.eqbuf));
    CK(cudaMemcpyAsync(diag, c.eqbuf, (size_t)c.neq * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    TRY(sync(c));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_get_diag");
}

extern "C" int pf_ebe_matvec(void **ctx, const int *prec, const double *p, double *u)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (!prec || !p || !u || !c.have_km || (*prec != 64 && *prec != 32 && *prec != 31 && *prec != 16) ||
        (c.kind != KIND_SOLID20 && *prec != 64) || (c.shared && *prec == 16)) {
        set_error("pf_ebe_matvec: invalid arguments or no storkm (8-node contexts: prec 64; "
                  "prec 16 needs per-element storkm)");
        return PF_FAILURE;
    }
    if (*prec == 16) TRY(ensure_km16(c));
    CK(cudaMemcpyAsync(c.eqbuf, p, (size_t)c.neq * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    TRY(launch_eq_to_slot(c, c.eqbuf, c.rres));
    TRY(launch_matvec(c, *prec, c.rres, c.u));
    TRY(check_kernel_error(c));
    TRY(launch_slot_to_eq(c, c.u, c.eqbuf));
    CK(cudaMemcpyAsync(u, c.eqbuf, (size_t)c.neq * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    TRY(sync(c));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_ebe_matvec");
}

// Mixed precision, restarted defect correction: each outer step solves
// K32 c = f - K64 x from c = 0 with FP32-storkm PCG, then x += c in FP64 and
// the FP64 true residual is recomputed.  Every restart discards the Krylov
// space, so the inner iterations add up to about twice the FP64 count.
static int solve_mixed_restart(Ctx &c, double tol, int limit, double ff, double *dev2)
{
    const double eta_min = 1e-5;   // inner relative tolerance floor
    const int max_outer = 50;
    CK(cudaMemsetAsync(c.x, 0, (size_t)c.nslots * sizeof(double), c.stream));
    CK(cudaMemcpyAsync(c.rres, c.f, (size_t)c.nslots * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    double rel = 1.0;
    int inner_total = 0, outer = 0, mv64 = 0;
    while (rel > tol && outer < max_outer && inner_total < limit) {
        ++outer;
        double eta = 0.5 * tol / rel;
        if (eta < eta_min) eta = eta_min;
        if (eta > 0.5) eta = 0.5;
        TRY(launch_pcg_init(c, c.rres, c.c, STOP_RELRES, eta, limit - inner_total));
        TRY(run_pcg(c, 32, c.c, limit - inner_total));
        inner_total += c.hst->iters;
        TRY(launch_axpy(c, c.x, c.c));
        TRY(true_relres(c, c.x, ff, &rel, dev2));
        ++mv64;
    }
    c.stats[0] = inner_total;
    c.stats[1] = outer;
    c.stats[3] = rel;
    c.stats[4] = mv64;
    c.stats[5] = inner_total;
    return 0;
}

// Mixed precision with residual replacement (the default mixed mode): one
// PCG run whose products use the FP32 storkm while x, r, p, d and every
// reduction stay FP64.  Whenever the recursive residual has dropped by
// `drop` since the last anchor, the FP64 true residual f - K64 x replaces it
// (defect correction) and the search direction is kept, so the Krylov space
// built so far is not thrown away.  The solve ends when the TRUE relative
// residual reaches tol.
static int solve_mixed(Ctx &c, double tol, int limit, double ff, double *dev2, int inner_prec)
{
    const double drop = 0.1;
    const int max_corrections = 200;
    double anchor = 1.0;                       // true relative residual at the last replacement
    double thr = anchor * drop > tol ? anchor * drop : tol;
    TRY(launch_pcg_init(c, c.f, c.x, STOP_RELRES, thr, limit));
    double rel = 1.0;
    int corrections = 0, mv64 = 0;
    for (;;) {
        TRY(pull_state(c));
        const int done = c.hst->iters;
        if (!c.hst->stop) TRY(run_pcg(c, inner_prec, c.x, limit - done));
        TRY(true_relres(c, c.x, ff, &rel, dev2));
        ++mv64;
        if (rel <= tol || c.hst->iters >= limit || corrections >= max_corrections) break;
        anchor = rel;
        thr = anchor * drop > tol ? anchor * drop : 0.5 * tol;
        TRY(launch_replace(c, thr));
        ++corrections;
    }
    c.stats[0] = c.hst->iters;
    c.stats[1] = corrections;
    c.stats[3] = rel;
    c.stats[4] = mv64;
    c.stats[5] = c.hst->iters;
    return 0;
}

extern "C" int pf_solve(void **ctx, const double *r, const double *tol, const int *limit, const int *mode,
                        double *xnew, int *iters, double *relres)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (!r || !tol || !limit || !mode || !xnew || !iters || !c.have_km || *limit < 1 ||
        (*mode != PF_MODE_P121 && *mode != PF_MODE_FP64_RES && *mode != PF_MODE_MIXED &&
         *mode != PF_MODE_MIXED_RESTART && *mode != PF_MODE_MIXED16)) {
        set_error("pf_solve: invalid arguments or no storkm");
        return PF_FAILURE;
    }
    if (c.kind != KIND_SOLID20 &&
        (*mode == PF_MODE_MIXED || *mode == PF_MODE_MIXED_RESTART || *mode == PF_MODE_MIXED16)) {
        set_error("pf_solve: the mixed modes need 20-node elements; 8-node contexts solve in FP64");
        return PF_FAILURE;
    }
    if (*mode == PF_MODE_MIXED16 && c.shared) {
        set_error("pf_solve: PF_MODE_MIXED16 needs per-element storkm (a shared km solves mixed with PF_MODE_MIXED)");
        return PF_FAILURE;
    }
    if (*mode == PF_MODE_MIXED16) TRY(ensure_km16(c));
    for (int i = 0; i < 8; ++i) c.stats[i] = 0.0;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double *dev2 = c.scr;
    CK(cudaMemcpyAsync(c.eqbuf, r, (size_t)c.neq * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    TRY(launch_eq_to_slot(c, c.eqbuf, c.f));
    CK(cudaEventRecord(e0, c.stream));
    int rc = 0;
    double ff = 0.0;
    {
        // f.f via the init kernel's r.r partial
        TRY(launch_pcg_init(c, c.f, c.x, *mode == PF_MODE_P121 ? STOP_CHECON : STOP_RELRES, *tol, *limit));
        TRY(pull_state(c));
        ff = c.hst->ff;
    }
    if (*mode == PF_MODE_MIXED || *mode == PF_MODE_MIXED16) {
        rc = solve_mixed(c, *tol, *limit, ff, dev2, *mode == PF_MODE_MIXED16 ? PREC_FP16_SYM : PREC_FP32_SYM);
    } else if (*mode == PF_MODE_MIXED_RESTART) {
        rc = solve_mixed_restart(c, *tol, *limit, ff, dev2);
    } else {
        rc = run_pcg(c, 64, c.x, *limit);
        c.stats[0] = c.hst->iters;
        c.stats[1] = 0;
        c.stats[3] = c.hst->metric;
        c.stats[4] = c.hst->iters;
    }
    if (rc) return PF_FAILURE;
    CK(cudaEventRecord(e1, c.stream));
    double rel = c.stats[3];
    if (*mode == PF_MODE_P121 || *mode == PF_MODE_FP64_RES)   // mixed modes end on a true residual
        TRY(true_relres(c, c.x, ff, &rel, dev2));
    float ms = 0.f;
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c.stats[2] = ms;
    c.stats[6] = rel;
    TRY(launch_slot_to_eq(c, c.x, c.eqbuf));
    CK(cudaMemcpyAsync(xnew, c.eqbuf, (size_t)c.neq * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    TRY(sync(c));
    *iters = (int)c.stats[0];
    if (relres) *relres = rel;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_solve");
}

extern "C" int pf_solve_stats(void **ctx, double *stats, const int *n)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp || !stats || !n) return PF_FAILURE;
    for (int i = 0; i < *n && i < 8; ++i) stats[i] = cp->stats[i];
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_solve_stats");
}

extern "C" int pf_bench_iterations(void **ctx, const int *prec, const int *steps, double *ms_total,
                                   double *ms_elem, double *ms_scatter)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (!prec || !steps || *steps < 1 || !c.have_km ||
        (*prec != 32 && *prec != 31 && *prec != 64 && *prec != 16) || (c.kind != KIND_SOLID20 && *prec != 64) ||
        (c.shared && *prec == 16)) {
        set_error("pf_bench_iterations: invalid arguments or no storkm (8-node contexts: prec 64; "
                  "prec 16 needs per-element storkm)");
        return PF_FAILURE;
    }
    if (*prec == 16) TRY(ensure_km16(c));
    const int n = *steps;
    // never-converging run on the resident load vector (tol 0, no limit hit)
    TRY(launch_pcg_init(c, c.f, c.c, STOP_RELRES, 0.0, n + 1));
    TRY(pull_state(c));
    if (c.hst->stop) {
        set_error("pf_bench_iterations: the resident load vector is zero (run pf_solve first)");
        return PF_FAILURE;
    }
    std::vector<cudaEvent_t> ev(3 * (size_t)n + 1);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    CK(cudaEventRecord(ev[0], c.stream));
    const bool tail = c.persistent && c.kind == KIND_SOLID20;
    for (int i = 0; i < n; ++i) {
        TRY(launch_elem(c, *prec, c.p));
        CK(cudaEventRecord(ev[3 * i + 1], c.stream));
        if (tail) {   // scatter, updates and finish in one persistent launch
            TRY(launch_pcg_tail(c, *prec, c.c));
            CK(cudaEventRecord(ev[3 * i + 2], c.stream));
        } else {
            TRY(launch_scatter(c, *prec, 0, c.p, c.u));
            CK(cudaEventRecord(ev[3 * i + 2], c.stream));
            TRY(launch_update1(c, c.c));
            TRY(launch_update2(c));
        }
        CK(cudaEventRecord(ev[3 * i + 3], c.stream));
    }
    CK(cudaStreamSynchronize(c.stream));
    TRY(check_kernel_error(c));
    double te = 0, ts = 0;
    for (int i = 0; i < n; ++i) {
        float a = 0, b = 0;
        CK(cudaEventElapsedTime(&a, ev[3 * i], ev[3 * i + 1]));
        CK(cudaEventElapsedTime(&b, ev[3 * i + 1], ev[3 * i + 2]));
        te += a;
        ts += b;
    }
    float tot = 0;
    CK(cudaEventElapsedTime(&tot, ev[0], ev[3 * (size_t)n]));
    for (auto &e : ev) cudaEventDestroy(e);
    if (ms_total) *ms_total = tot;
    if (ms_elem) *ms_elem = te;
    if (ms_scatter) *ms_scatter = ts;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_bench_iterations");
}

extern "C" int pf_centroid_stress(void **ctx, const int *iel, const double *xnew, double *sigma)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (c.kind != KIND_SOLID20) {
        set_error("pf_centroid_stress: needs a 20-node context (pf_setup)");
        return PF_FAILURE;
    }
    if (!iel || !xnew || !sigma || *iel < 1 || *iel > c.nels || c.nmat == 0) {
        set_error("pf_centroid_stress: invalid element or no material");
        return PF_FAILURE;
    }
    double *sig = c.scr + 2;
    CK(cudaMemcpyAsync(c.eqbuf, xnew, (size_t)c.neq * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    TRY(launch_eq_to_slot(c, c.eqbuf, c.rres));
    TRY(launch_centroid_stress(c, *iel - 1, 1, c.rres, sig));
    CK(cudaMemcpyAsync(sigma, sig, 6 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    TRY(sync(c));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_centroid_stress");
}

extern "C" int pf_element_stresses(void **ctx, const double *xnew, const int *first, const int *count,
                                   double *sigma)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    Ctx &c = *cp;
    if (c.kind != KIND_SOLID20) {
        set_error("pf_element_stresses: needs a 20-node context (pf_setup)");
        return PF_FAILURE;
    }
    if (!xnew || !first || !count || !sigma || *first < 1 || *count < 0 || *first - 1 + (long long)*count > c.nels ||
        c.nmat == 0) {
        set_error("pf_element_stresses: invalid element range or no material");
        return PF_FAILURE;
    }
    if (*count == 0) return PF_SUCCESS;
    double *sig = (double *)c.utemp;   // 6 x count <= 60 x nels doubles
    CK(cudaMemcpyAsync(c.eqbuf, xnew, (size_t)c.neq * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    TRY(launch_eq_to_slot(c, c.eqbuf, c.rres));
    TRY(launch_centroid_stress(c, *first - 1, *count, c.rres, sig));
    CK(cudaMemcpyAsync(sigma, sig, (size_t)6 * *count * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    TRY(sync(c));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_element_stresses");
}

extern "C" int pf_tuning(void **ctx, int *warps, int *stages, float *ms)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp || !warps || !stages || !ms) return PF_FAILURE;
    *warps = cp->sym_warps;
    *stages = cp->sym_stages;
    for (int i = 0; i < 3; ++i) ms[i] = cp->tune_ms[i];
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_tuning");
}

extern "C" int pf_tuning16(void **ctx, int *warps, int *stages, float *ms)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp || !warps || !stages || !ms) return PF_FAILURE;
    if (!cp->km16_ok) {
        set_error("pf_tuning16: the FP16 storkm has not been packed (no FP16 product yet)");
        return PF_FAILURE;
    }
    if (h16_config(cp->h16_cfg, warps, stages)) return PF_FAILURE;
    for (int i = 0; i < 3; ++i) ms[i] = cp->tune16_ms[i];
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_tuning16");
}

extern "C" int pf_set_tuning(void **ctx, const int *config)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp || !config) return PF_FAILURE;
    Ctx &c = *cp;
    if (*config < -1 || *config > 2) {
        set_error("pf_set_tuning: configuration %d is not in -1..2", *config);
        return PF_FAILURE;
    }
    if (!c.km32p) {
        set_error("pf_set_tuning: form or set storkm first");
        return PF_FAILURE;
    }
    if (*config == -1) {
        TRY(autotune_sym32(c, c.x));
        return PF_SUCCESS;
    }
    set_sym_config(c, *config);
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_set_tuning");
}

extern "C" int pf_check_wait_timeout(void **ctx, const int *polls)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    if (!polls || *polls < 1) {
        set_error("pf_check_wait_timeout: *polls must be at least 1");
        return PF_FAILURE;
    }
    TRY(launch_wait_probe(*cp, *polls));
    if (check_kernel_error(*cp)) return PF_FAILURE;   // the timeout, reported as the kernels report it
    set_error("pf_check_wait_timeout: the wait completed, so the timeout path did not run");
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_check_wait_timeout");
}

extern "C" int pf_set_persistent(void **ctx, const int *on)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp) return PF_FAILURE;
    if (!on) {
        set_error("pf_set_persistent: null argument");
        return PF_FAILURE;
    }
    cp->persistent = *on != 0;
    drop_graph(*cp);
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_set_persistent");
}

extern "C" int pf_set_graphs(void **ctx, const int *on)
try {
    Ctx *cp = get_ctx(ctx);
    if (!cp || !on) return PF_FAILURE;
    cp->use_graphs = *on != 0;
    if (!cp->use_graphs) drop_graph(*cp);
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_set_graphs");
}

extern "C" int pf_kernel_launches(void **ctx, long long *count)
try {
    if (!count) return PF_FAILURE;
    *count = g_xx3_launches;
    if (ctx && *ctx) *count += ((Ctx *)*ctx)->launches;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_kernel_launches");
}
