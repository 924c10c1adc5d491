// fit_capi.cu -- extern "C" entry points of libwakis_fit.so (declared in include/wakis_fit.h).
//
// A context owns: the coefficient arrays in the field dtype, the 1-D metric arrays, the
// source / tap tables, a private non-blocking stream on which every kernel is issued
// (ordered after and before the caller's stream with events, so caller writes to the
// fields and our kernels never race), and the CUDA graphs of fit_run.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "wakis_fit.h"
#include "fit_kernels.cuh"
#include "fit_tma.cuh"

using namespace fit;

namespace {

std::atomic<long long> g_launches{0};
std::mutex g_err_mu;
std::string g_create_error;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct FitCtx {
    int device = 0;
    int dtype = FIT_F32;
    int use_cond = 0;
    Geom g{};
    int bc_lo[3]{}, bc_hi[3]{};
    int edits[6]{};
    int n_edits = 0;
    void *E = nullptr, *H = nullptr, *J = nullptr;
    cudaStream_t user = nullptr;  // caller stream (may be the legacy default stream)
    cudaStream_t own = nullptr;   // private stream all kernels run on
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    // metrics: FP64 (coefficient build) and field-dtype copies (stencil)
    double* dL[3]{};
    double* dtL0[3]{};  // unedited dual lengths
    void* tL_T[3]{};
    void* L_T[3]{};
    bool metrics_set = false;
    // coefficients
    void *ch = nullptr, *ce = nullptr, *cl = nullptr, *cj = nullptr, *sg = nullptr;
    bool coeffs_set = false;
    bool explicit_ready = false;
    double dt = 0.0;
    // beam
    BeamArgs beam{};
    double* d_beam_z = nullptr;
    double* d_beam_dtieps = nullptr;
    std::vector<double> ieps_line;
    double beam_vt = 0.0;
    double* d_vt_table = nullptr;
    long long vt_len = 0;
    // plane source
    PlaneArgs plane{};
    double *d_prof = nullptr, *d_c1 = nullptr, *d_c2 = nullptr, *d_gt = nullptr, *d_stash = nullptr;
    // abc
    int abc_axes = 0;
    // wake taps
    TapArgs tap{};
    long long *d_base = nullptr, *d_row = nullptr;
    int *d_em = nullptr, *d_ek0 = nullptr, *d_ecnt = nullptr;
    double *d_dz = nullptr, *d_acc = nullptr, *d_comp = nullptr, *d_scratch = nullptr;
    double *d_wp3d = nullptr, *d_wpx = nullptr, *d_wpy = nullptr;
    // step counter and graphs
    long long* d_step = nullptr;
    cudaGraphExec_t graph = nullptr;
    long long graph_chunk = 0;
    bool capturing = false;
    int* d_err = nullptr;   // device error word written by kernels (FIT_ERR_TIMEOUT)
    int nsm = 1;            // SM count: grid of the persistent staged kernels
    bool staged = false;    // staged (bulk-copy) passes when the grid is aligned (opt-in)
    bool fused = false;     // fused single-pass step in device loops (ping-pong with E2/H2)
    void *E2 = nullptr, *H2 = nullptr;  // the second field buffers of the fused step
    int fused_vec = 4, fused_rows = 8, fused_zseg = 1, fused_ctas = 2;  // tile shape of the fused step
    int fused_staging = 0;  // 0: loads; 1, 2: TMA plane rings (fit_set_fused_staging)
    long long wait_limit = kWaitLimit;  // polls of the bounded waits for data (fit_set_wait_limit)
    int tma_prefetch = 1;  // planes the TMA-fed step's L2 prefetch runs ahead of its ring loads
    bool graph_fused = false;  // the cached graph holds fused steps
    unsigned short* d_code = nullptr;  // coded coefficients: one code per cell (nullptr: dense)
    void* d_tab = nullptr;             // [code][ch, ce, cl][x, y, z, pad] in the field dtype
    int ncodes = 0;
    RecordArgs rec{};           // Ez line history of recorded steps (nlines = 0: off)
    JRecordArgs jrec{};         // Jz line history of recorded steps (nlines = 0: off)
    double* d_jsig = nullptr;   // sigma_z on the Jz record lines
    MonitorArgs mon{};          // field monitor epilogue of device-loop steps (nf = 0: off)
    double2* d_mon_phases = nullptr;
    std::atomic<bool> in_pool{false};  // submitted to a FitPool and not yet reported done
    std::string err;
};

namespace {

int fail(FitCtx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) {
        c->err = buf;
    } else {
        std::lock_guard<std::mutex> lk(g_err_mu);
        g_create_error = buf;
    }
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(c, FIT_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));     \
    } while (0)

size_t esize(const FitCtx* c) { return c->dtype == FIT_F64 ? 8 : 4; }

// Device buffers are stream-ordered allocations (cudaMallocAsync / cudaFreeAsync) on the
// context stream: a plain cudaFree waits for the whole device, including the kernels of
// other contexts and of a serving pool, while the stream-ordered calls wait for nothing.
// The device's default memory pool keeps freed blocks for reuse (release threshold set
// to the maximum once per device), like a caching allocator.
void keep_freed_blocks(int device) {
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), device) != done.end()) return;
    cudaMemPool_t mp;
    if (cudaDeviceGetDefaultMemPool(&mp, device) == cudaSuccess) {
        uint64_t thr = ~0ull;
        cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    done.push_back(device);
}

int dev_alloc(FitCtx* c, void** p, size_t bytes) {
    if (*p) {
        cudaFreeAsync(*p, c->own);
        *p = nullptr;
    }
    if (bytes == 0) return FIT_OK;
    cudaError_t e = cudaMallocAsync(p, bytes, c->own);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(c, e == cudaErrorMemoryAllocation ? FIT_ERR_NOMEM : FIT_ERR_CUDA,
                    "cudaMallocAsync(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    return FIT_OK;
}

template <typename P>
int upload(FitCtx* c, P** dst, const void* src, size_t bytes) {
    int rc = dev_alloc(c, reinterpret_cast<void**>(dst), bytes);
    if (rc) return rc;
    if (bytes) CK(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, c->own));
    return FIT_OK;
}

void dfree(void* p, cudaStream_t st) {
    if (p) cudaFreeAsync(p, st);
}

// ordering with the caller's stream
int enter(FitCtx* c) {
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    CK(cudaSetDevice(c->device));
    CK(cudaEventRecord(c->ev_in, c->user));
    CK(cudaStreamWaitEvent(c->own, c->ev_in, 0));
    return FIT_OK;
}
int leave(FitCtx* c) {
    CK(cudaGetLastError());
    CK(cudaEventRecord(c->ev_out, c->own));
    CK(cudaStreamWaitEvent(c->user, c->ev_out, 0));
    return FIT_OK;
}

// the Jz record arguments of a launch: the beam as it is for this step
JRecordArgs jrec_args(const FitCtx* c) {
    JRecordArgs j = c->jrec;
    if (j.nlines > 0) {
        j.beam = c->beam;
        j.vt_table = c->d_vt_table;
        j.vt_len = c->vt_len;
        j.vt_host = c->beam_vt;
    }
    return j;
}

int pick_vec(const FitCtx* c) {
    const int nx = c->g.nx;
    if (c->dtype == FIT_F32) return (nx % 4 == 0) ? 4 : (nx % 2 == 0 ? 2 : 1);
    return (nx % 2 == 0) ? 2 : 1;
}

template <typename T>
Metric<T> metric(const FitCtx* c) {
    Metric<T> m;
    for (int a = 0; a < 3; ++a) {
        m.L[a] = static_cast<const T*>(c->L_T[a]);
        m.tL[a] = static_cast<const T*>(c->tL_T[a]);
    }
    return m;
}

unsigned grid1d(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

void count(const FitCtx* c, long long k = 1) {
    if (!c->capturing) g_launches += k;
}

// any change of what a captured step launches drops the graph
void invalidate(FitCtx* c) {
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
}

// back to dense coefficients (the cached graph may hold coded launches)
void drop_codes(FitCtx* c) {
    if (!c->d_code) return;
    invalidate(c);
    dfree(c->d_code, c->own);
    dfree(c->d_tab, c->own);
    c->d_code = nullptr;
    c->d_tab = nullptr;
    c->ncodes = 0;
}

int launches_per_step(const FitCtx* c) {
    int n = 3 + (c->mon.nf > 0);
    for (int a = 0; a < 3; ++a) n += (c->abc_axes >> a) & 1;
    return n;
}

// staged kernels need 16-byte aligned stream starts: Nx*sizeof(T) % 16 == 0
bool staged_ok(const FitCtx* c) { return c->staged && ((long long)c->g.nx * (long long)esize(c)) % 16 == 0; }

// pipeline stages and threads per CTA of the staged passes (one CTA per SM)
constexpr int kNstH = 2, kTpbH = 512, kNstE = 2, kTpbE = 384;

template <typename T, int VEC, int NS, int NST, int TPB>
size_t staged_bytes() {
    return (size_t)NST * ((size_t)NS * TPB * VEC + 2 * (16 / sizeof(T))) * sizeof(T) + NST * sizeof(unsigned long long);
}

template <typename KernelPtr>
void allow_smem(KernelPtr k, size_t bytes) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// vectors between a thread and its counterpart in the next resident wave of CTAs of a
// coded two-pass kernel (its L2 prefetch distance); 0 turns the prefetch off.  The
// single-cell kernels go without: their prefetch did not pay in the serving pool (the
// cell-pair kernels have their own, pair_ahead).
#ifndef FIT_TWO_PASS_PREFETCH
#define FIT_TWO_PASS_PREFETCH 1
#endif
template <typename T, int VEC>
long long coded_ahead(const FitCtx* c, bool e_pass) {
    if (VEC < 2 || !FIT_TWO_PASS_PREFETCH) return 0;
    // resident CTAs per SM of each kernel, queried once (no stream work: safe during capture)
    static const int occ_h = [] {
        int o = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_hpass_coded<T, VEC>, 256, 0) == cudaSuccess ? o : 0;
    }();
    static const int occ_e = [] {
        int o = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_epass_coded<T, VEC, 1>, 256, 0) == cudaSuccess ? o
                                                                                                              : 0;
    }();
    const int occ = e_pass ? occ_e : occ_h;
    return occ > 0 ? (long long)c->nsm * occ * 256 : 0;
}

// the same for the cell-pair kernels (Nx odd, N even)
template <typename T>
long long pair_ahead(const FitCtx* c, bool e_pass) {
    if (!FIT_TWO_PASS_PREFETCH) return 0;
    static const int occ_h = [] {
        int o = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_hpass_pair<T>, 256, 0) == cudaSuccess ? o : 0;
    }();
    static const int occ_e = [] {
        int o = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_epass_pair<T, 1>, 256, 0) == cudaSuccess ? o : 0;
    }();
    const int occ = e_pass ? occ_e : occ_h;
    return occ > 0 ? (long long)c->nsm * occ * 256 : 0;
}

// coded grids with Nx odd and N even step cell pairs instead of single cells
template <int VEC>
bool use_pairs(const FitCtx* c) {
    return VEC == 1 && c->d_code && c->d_tab && c->g.N % 2 == 0;
}

template <typename T, int VEC>
void launch_h(FitCtx* c) {
    if (VEC * sizeof(T) == 16 && staged_ok(c)) {
        const size_t sm = staged_bytes<T, VEC, 13, kNstH, kTpbH>();
        auto k = k_hpass_staged<T, VEC, kNstH, kTpbH>;
        allow_smem(k, sm);
        k<<<c->nsm, kTpbH, sm, c->own>>>(static_cast<const T*>(c->E), static_cast<T*>(c->H),
                                       static_cast<const T*>(c->ch), c->g, metric<T>(c), c->d_err, c->wait_limit);
    } else if (use_pairs<VEC>(c)) {
        k_hpass_pair<T><<<grid1d(c->g.N / 2, 256), 256, 0, c->own>>>(static_cast<const T*>(c->E), static_cast<T*>(c->H),
                                                                     c->g, metric<T>(c), c->d_code,
                                                                     static_cast<const T*>(c->d_tab),
                                                                     pair_ahead<T>(c, false));
    } else if (c->d_code) {
        const long long nv = c->g.N / VEC;
        k_hpass_coded<T, VEC><<<grid1d(nv, 256), 256, 0, c->own>>>(static_cast<const T*>(c->E),
                                                                   static_cast<T*>(c->H), c->g, metric<T>(c),
                                                                   c->d_code, static_cast<const T*>(c->d_tab),
                                                                   coded_ahead<T, VEC>(c, false));
    } else {
        const long long nv = c->g.N / VEC;
        k_hpass<T, VEC><<<grid1d(nv, 256), 256, 0, c->own>>>(static_cast<const T*>(c->E), static_cast<T*>(c->H),
                                                             static_cast<const T*>(c->ch), c->g, metric<T>(c));
    }
    count(c);
}

template <typename T, int VEC>
void launch_e(FitCtx* c, int mode, const StepArgs& st) {
    T* E = static_cast<T*>(c->E);
    const T* H = static_cast<const T*>(c->H);
    const T* ce = static_cast<const T*>(c->ce);
    const T* cl = static_cast<const T*>(c->cl);
    T* J = static_cast<T*>(c->J);
    const T* cj = static_cast<const T*>(c->cj);
    const T* sg = static_cast<const T*>(c->sg);
    if (VEC * sizeof(T) == 16 && staged_ok(c) && mode != 2) {
        if (mode == 1) {
            const size_t sm = staged_bytes<T, VEC, 16, kNstE, kTpbE>();
            auto k = k_epass_staged<T, VEC, kNstE, 1, kTpbE>;
            allow_smem(k, sm);
            k<<<c->nsm, kTpbE, sm, c->own>>>(E, H, ce, cl, J, c->use_cond, c->g, metric<T>(c), c->beam, c->plane, st,
                                           c->d_err, c->wait_limit);
        } else {
            const size_t sm = staged_bytes<T, VEC, 13, kNstE, kTpbE>();
            auto k = k_epass_staged<T, VEC, kNstE, 0, kTpbE>;
            allow_smem(k, sm);
            k<<<c->nsm, kTpbE, sm, c->own>>>(E, H, ce, cl, J, c->use_cond, c->g, metric<T>(c), c->beam, c->plane, st,
                                           c->d_err, c->wait_limit);
        }
        count(c);
        return;
    }
    const long long nv = c->g.N / VEC;
    const unsigned nb = grid1d(nv, 256);
    const T* tab = static_cast<const T*>(c->d_tab);
    if (use_pairs<VEC>(c) && mode != 2) {
        const unsigned np = grid1d(c->g.N / 2, 256);
        if (mode == 1)
            k_epass_pair<T, 1><<<np, 256, 0, c->own>>>(E, H, J, c->use_cond, c->g, metric<T>(c), c->beam, c->plane, st,
                                                       c->d_code, tab, pair_ahead<T>(c, true));
        else
            k_epass_pair<T, 0><<<np, 256, 0, c->own>>>(E, H, J, c->use_cond, c->g, metric<T>(c), c->beam, c->plane, st,
                                                       c->d_code, tab, pair_ahead<T>(c, true));
        count(c);
        return;
    }
    if (c->d_code && mode == 0)
        k_epass_coded<T, VEC, 0><<<nb, 256, 0, c->own>>>(E, H, J, c->use_cond, c->g, metric<T>(c), c->beam, c->plane,
                                                         st, c->d_code, tab, coded_ahead<T, VEC>(c, true));
    else if (c->d_code && mode == 1)
        k_epass_coded<T, VEC, 1><<<nb, 256, 0, c->own>>>(E, H, J, c->use_cond, c->g, metric<T>(c), c->beam, c->plane,
                                                         st, c->d_code, tab, coded_ahead<T, VEC>(c, true));
    else if (mode == 0)
        k_epass<T, VEC, 0><<<nb, 256, 0, c->own>>>(E, H, ce, cl, J, cj, sg, c->use_cond, c->g, metric<T>(c), c->beam, c->plane, st);
    else if (mode == 1)
        k_epass<T, VEC, 1><<<nb, 256, 0, c->own>>>(E, H, ce, cl, J, cj, sg, c->use_cond, c->g, metric<T>(c), c->beam, c->plane, st);
    else
        k_epass<T, VEC, 2><<<nb, 256, 0, c->own>>>(E, H, ce, cl, J, cj, sg, c->use_cond, c->g, metric<T>(c), c->beam, c->plane, st);
    count(c);
}

// the field-monitor epilogue of a step whose new E is in E (device loop: step number
// from the counter; host step: n)
template <typename T>
void launch_monitor(FitCtx* c, const T* E, bool device_step, long long n) {
    if (c->mon.nf <= 0) return;
    const long long n3 = 3 * c->g.N;
    const unsigned grid = (unsigned)std::min<long long>(grid1d(n3, 256), 8LL * c->nsm);
    k_monitor<T><<<grid, 256, 0, c->own>>>(E, c->g.N, c->mon, device_step ? c->d_step : nullptr,
                                          device_step ? -1 : n);
    count(c);
}

template <typename T>
void launch_step_t(FitCtx* c, long long n, int mode, bool device_step) {
    StepArgs st{};
    if (device_step) {
        st.d_step = c->d_step;
        st.vt_table = c->d_vt_table;
        st.vt_len = c->vt_len;
    } else {
        st.n = n;
        st.vt = c->beam_vt;
    }
    const bool need_pro =
        device_step || c->plane.active || c->tap.nlines > 0 || c->rec.nlines > 0 || c->jrec.nlines > 0;
    if (need_pro) {
        k_prologue<T><<<1, 512, 0, c->own>>>(static_cast<T*>(c->E), static_cast<T*>(c->H), c->g, c->plane, c->tap,
                                             n, device_step ? c->d_step : nullptr, c->rec, jrec_args(c));
        count(c);
    }
    const int vec = pick_vec(c);
    if (vec == 4) {
        if constexpr (sizeof(T) == 4) {
            launch_h<T, 4>(c);
            launch_e<T, 4>(c, mode, st);
        }
    } else if (vec == 2) {
        launch_h<T, 2>(c);
        launch_e<T, 2>(c, mode, st);
    } else {
        launch_h<T, 1>(c);
        launch_e<T, 1>(c, mode, st);
    }
    for (int a = 0; a < 3; ++a) {
        if (c->abc_axes & (1 << a)) {
            const int pa = a == 0 ? c->g.ny : c->g.nx;
            const int pb = a == 2 ? c->g.ny : c->g.nz;
            k_abc_lo<T><<<grid1d(6LL * pa * pb, 256), 256, 0, c->own>>>(static_cast<T*>(c->E), static_cast<T*>(c->H),
                                                                     c->g, a);
            count(c);
        }
    }
    launch_monitor<T>(c, static_cast<const T*>(c->E), device_step, n);
}

void launch_step(FitCtx* c, long long n, int mode, bool device_step) {
    if (c->dtype == FIT_F64)
        launch_step_t<double>(c, n, mode, device_step);
    else
        launch_step_t<float>(c, n, mode, device_step);
}

// the fused step serves the elided-J device loop without plane sources or ABC updates,
// on grids with Nx a multiple of the 2- or 4-wide vector
bool fused_ok(const FitCtx* c, int mode) {
    return c->fused && c->E2 && c->H2 && mode != 2 && !c->plane.active && !c->abc_axes && pick_vec(c) >= 2;
}

template <typename T, int VEC, int FY, int MB>
void launch_fused_shape(FitCtx* c, int mode, const StepArgs& st, bool forward, const BeamArgs& beam) {
    constexpr int FX = 32 * VEC;
    const T* Ein = static_cast<const T*>(forward ? c->E : c->E2);
    const T* Hin = static_cast<const T*>(forward ? c->H : c->H2);
    T* Eout = static_cast<T*>(forward ? c->E2 : c->E);
    T* Hout = static_cast<T*>(forward ? c->H2 : c->H);
    const int zlen = (c->g.nz + c->fused_zseg - 1) / c->fused_zseg;
    const dim3 grid((unsigned)((c->g.nx + FX - 1) / FX), (unsigned)((c->g.ny + FY - 1) / FY),
                    (unsigned)((c->g.nz + zlen - 1) / zlen));
    const dim3 block(32, FY + 1);
    const T* ch = static_cast<const T*>(c->ch);
    const T* ce = static_cast<const T*>(c->ce);
    const T* cl = static_cast<const T*>(c->cl);
    T* J = static_cast<T*>(c->J);
    const unsigned short* code = c->d_code;
    const T* tab = static_cast<const T*>(c->d_tab);
    if (mode == 1 && code) {
        k_step_fused<T, VEC, FY, MB, 1, true><<<grid, block, 0, c->own>>>(
            Ein, Hin, Eout, Hout, ch, ce, cl, J, c->use_cond, c->g, metric<T>(c), beam, st, zlen, code, tab);
    } else if (code) {
        k_step_fused<T, VEC, FY, MB, 0, true><<<grid, block, 0, c->own>>>(
            Ein, Hin, Eout, Hout, ch, ce, cl, J, c->use_cond, c->g, metric<T>(c), beam, st, zlen, code, tab);
    } else {
        if (mode == 1)
            k_step_fused<T, VEC, FY, MB, 1, false><<<grid, block, 0, c->own>>>(
                Ein, Hin, Eout, Hout, ch, ce, cl, J, c->use_cond, c->g, metric<T>(c), beam, st, zlen, nullptr,
                nullptr);
        else
            k_step_fused<T, VEC, FY, MB, 0, false><<<grid, block, 0, c->own>>>(
                Ein, Hin, Eout, Hout, ch, ce, cl, J, c->use_cond, c->g, metric<T>(c), beam, st, zlen, nullptr,
                nullptr);
    }
    count(c);
}

// the fused step in the context's tile shape: fused_vec cells per thread, fused_rows rows,
// register budget for fused_ctas CTAs per SM (8 rows: 2; 4 rows: 3 or 4).  Budgets of 5
// or 6 CTAs per SM with 4 rows and 3 with 8 rows were timed for the coded step on the
// 512x512x1024 pillbox (2.99 ms and more against 2.89 ms) and are not compiled.
template <typename T, int VEC>
void launch_fused_vec(FitCtx* c, int mode, const StepArgs& st, bool forward, const BeamArgs& beam) {
    if (c->fused_rows == 8)
        launch_fused_shape<T, VEC, 8, 2>(c, mode, st, forward, beam);
    else if (c->fused_ctas == 4)
        launch_fused_shape<T, VEC, 4, 4>(c, mode, st, forward, beam);
    else
        launch_fused_shape<T, VEC, 4, 3>(c, mode, st, forward, beam);
}

// ---------------------------------------------------------------- TMA-fed fused step
PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// the grids the TMA-fed step serves: coded coefficients, every box row and plane stride
// a multiple of 16 bytes (Nx a multiple of 8 for the 2-byte codes), the widest vector
bool tma_grid_ok(const FitCtx* c) {
    return c->d_code && c->g.nx % 8 == 0 && (c->dtype == FIT_F64 || c->fused_vec == 4);
}

// 4-D map (Nx, Ny, Nz, 3 components) of a field buffer, box (bw, bh, 1, 3)
bool encode_field_map(CUtensorMap* m, const FitCtx* c, const void* base, int bw, int bh) {
    const auto enc = tmap_encoder();
    if (!enc || !base) return false;
    const cuuint64_t es = esize(c);
    const cuuint64_t dims[4] = {(cuuint64_t)c->g.nx, (cuuint64_t)c->g.ny, (cuuint64_t)c->g.nz, 3};
    const cuuint64_t strides[3] = {dims[0] * es, dims[0] * dims[1] * es, (cuuint64_t)c->g.N * es};
    const cuuint32_t box[4] = {(cuuint32_t)bw, (cuuint32_t)bh, 1, 3};
    const cuuint32_t elem[4] = {1, 1, 1, 1};
    return enc(m, c->dtype == FIT_F64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
               const_cast<void*>(base), dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 3-D map (Nx, Ny, Nz) of the 16-bit coefficient codes, box (bw, bh, 1)
bool encode_code_map(CUtensorMap* m, const FitCtx* c, int bw, int bh) {
    const auto enc = tmap_encoder();
    if (!enc || !c->d_code) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)c->g.nx, (cuuint64_t)c->g.ny, (cuuint64_t)c->g.nz};
    const cuuint64_t strides[2] = {dims[0] * 2, dims[0] * dims[1] * 2};
    const cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
    const cuuint32_t elem[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, c->d_code, dims, strides, box, elem,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the three maps of one step direction for the tile shape (FY rows)
template <typename T, int VEC, int FY, int NE, int NH>
bool encode_step_maps(const FitCtx* c, bool forward, CUtensorMap* mE, CUtensorMap* mH, CUtensorMap* mC) {
    using L = TmaLayout<T, VEC, FY, NE, NH>;
    return encode_field_map(mE, c, forward ? c->E : c->E2, L::EW, L::ER) &&
           encode_field_map(mH, c, forward ? c->H : c->H2, L::HW, L::HR) && encode_code_map(mC, c, L::CW, L::HR);
}

// returns false (nothing launched) when the maps cannot be encoded
template <typename T, int VEC, int FY, int MB, int NE, int NH>
bool launch_tma_shape(FitCtx* c, int mode, const StepArgs& st, bool forward, const BeamArgs& beam) {
    using L = TmaLayout<T, VEC, FY, NE, NH>;
    CUtensorMap mE, mH, mC;
    if (!encode_step_maps<T, VEC, FY, NE, NH>(c, forward, &mE, &mH, &mC)) return false;
    const T* Ein = static_cast<const T*>(forward ? c->E : c->E2);
    const T* Hin = static_cast<const T*>(forward ? c->H : c->H2);
    T* Eout = static_cast<T*>(forward ? c->E2 : c->E);
    T* Hout = static_cast<T*>(forward ? c->H2 : c->H);
    const int zlen = (c->g.nz + c->fused_zseg - 1) / c->fused_zseg;
    const dim3 grid((unsigned)((c->g.nx + L::FX - 1) / L::FX), (unsigned)((c->g.ny + FY - 1) / FY),
                    (unsigned)((c->g.nz + zlen - 1) / zlen));
    const dim3 block(32, FY + 1);
    const T* tab = static_cast<const T*>(c->d_tab);
    T* J = static_cast<T*>(c->J);
    if (mode == 1) {
        auto k = k_step_tma<T, VEC, FY, MB, 1, NE, NH>;
        allow_smem(k, L::BYTES);
        k<<<grid, block, L::BYTES, c->own>>>(mE, mH, mC, Ein, Hin, Eout, Hout, J, c->use_cond, c->g, metric<T>(c),
                                             beam, st, zlen, c->d_code, tab, c->d_err, c->wait_limit,
                                             c->tma_prefetch);
    } else {
        auto k = k_step_tma<T, VEC, FY, MB, 0, NE, NH>;
        allow_smem(k, L::BYTES);
        k<<<grid, block, L::BYTES, c->own>>>(mE, mH, mC, Ein, Hin, Eout, Hout, J, c->use_cond, c->g, metric<T>(c),
                                             beam, st, zlen, c->d_code, tab, c->d_err, c->wait_limit,
                                             c->tma_prefetch);
    }
    count(c);
    return true;
}

// tile shapes (rows, CTAs per SM, E ring depth, H ring depth): 4 rows and 3 CTAs per SM
// with rings of 4 / 2 planes (staging 1); 4 rows and 4 CTAs per SM with 3 / 2 (staging
// 2, shared memory and registers sized for four); 8 rows, 2 CTAs per SM, 3 / 2
template <typename T, int VEC>
bool launch_tma(FitCtx* c, int mode, const StepArgs& st, bool forward, const BeamArgs& beam) {
    if (c->fused_rows == 8) return launch_tma_shape<T, VEC, 8, 2, 3, 2>(c, mode, st, forward, beam);
    if (c->fused_staging == 2) return launch_tma_shape<T, VEC, 4, 4, 3, 2>(c, mode, st, forward, beam);
    return launch_tma_shape<T, VEC, 4, 3, 4, 2>(c, mode, st, forward, beam);
}

template <typename T, int VEC>
bool tma_maps_ok_t(const FitCtx* c, int staging, int rows, bool forward) {
    CUtensorMap a, b, d;
    if (rows == 8) return encode_step_maps<T, VEC, 8, 3, 2>(c, forward, &a, &b, &d);
    if (staging == 2) return encode_step_maps<T, VEC, 4, 3, 2>(c, forward, &a, &b, &d);
    return encode_step_maps<T, VEC, 4, 4, 2>(c, forward, &a, &b, &d);
}

bool tma_maps_ok(const FitCtx* c, int staging, int rows) {
    for (int f = 0; f < 2; ++f) {
        const bool ok = c->dtype == FIT_F64 ? tma_maps_ok_t<double, 2>(c, staging, rows, f == 0)
                                            : tma_maps_ok_t<float, 4>(c, staging, rows, f == 0);
        if (!ok) return false;
    }
    return true;
}

void launch_fused(FitCtx* c, int mode, const StepArgs& st, bool forward, const BeamArgs& beam) {
    if (c->fused_staging && tma_grid_ok(c)) {
        const bool done = c->dtype == FIT_F64 ? launch_tma<double, 2>(c, mode, st, forward, beam)
                                              : launch_tma<float, 4>(c, mode, st, forward, beam);
        if (done) return;  // else the load-fed kernel (same results)
    }
    if (c->dtype == FIT_F64)
        launch_fused_vec<double, 2>(c, mode, st, forward, beam);
    else if (c->fused_vec == 4)
        launch_fused_vec<float, 4>(c, mode, st, forward, beam);
    else
        launch_fused_vec<float, 2>(c, mode, st, forward, beam);
}

// default tile shape: the widest vector, 8 rows, z ranges for about four waves
void fused_default_shape(FitCtx* c) {
    c->fused_vec = pick_vec(c) == 4 ? 4 : 2;
    c->fused_rows = 8;
    c->fused_ctas = 2;
    const long long tiles = (long long)((c->g.nx + 32 * c->fused_vec - 1) / (32 * c->fused_vec)) *
                            ((c->g.ny + c->fused_rows - 1) / c->fused_rows);
    const long long want = (4LL * 2 * c->nsm + tiles - 1) / tiles;
    c->fused_zseg = (int)std::max<long long>(1, std::min<long long>(want, std::max(1, c->g.nz / 8)));
}

// one fused step: (E, H) -> (E2, H2) when forward, else back; the prologue (wake taps,
// step counter) reads the step's input buffer
void launch_fused_step(FitCtx* c, int mode, bool forward, const StepArgs& st, long long n) {
    const bool dev = st.d_step != nullptr;
    if (c->dtype == FIT_F64) {
        k_prologue<double><<<1, 512, 0, c->own>>>(static_cast<double*>(forward ? c->E : c->E2),
                                                   static_cast<double*>(forward ? c->H : c->H2), c->g, c->plane, c->tap,
                                                   n, dev ? c->d_step : nullptr, c->rec, jrec_args(c));
        count(c);
        launch_fused(c, mode, st, forward, c->beam);
        launch_monitor<double>(c, static_cast<const double*>(forward ? c->E2 : c->E), dev, n);
    } else {
        k_prologue<float><<<1, 512, 0, c->own>>>(static_cast<float*>(forward ? c->E : c->E2),
                                                 static_cast<float*>(forward ? c->H : c->H2), c->g, c->plane, c->tap,
                                                 n, dev ? c->d_step : nullptr, c->rec, jrec_args(c));
        count(c);
        launch_fused(c, mode, st, forward, c->beam);
        launch_monitor<float>(c, static_cast<const float*>(forward ? c->E2 : c->E), dev, n);
    }
}

StepArgs device_step_args(const FitCtx* c) {
    StepArgs st{};
    st.d_step = c->d_step;
    st.vt_table = c->d_vt_table;
    st.vt_len = c->vt_len;
    return st;
}

int check_ready(FitCtx* c) {
    if (!c) return FIT_ERR_ARG;
    if (!c->metrics_set) return fail(c, FIT_ERR_STATE, "fit_set_metrics has not been called");
    if (!c->coeffs_set) return fail(c, FIT_ERR_STATE, "fit_set_coeffs has not been called");
    if (!c->E || !c->H || !c->J) return fail(c, FIT_ERR_STATE, "field pointers are not set");
    return FIT_OK;
}

// one pass of the code build in the field dtype (kernels k_code_*)
template <typename T>
int build_codes_t(FitCtx* c, int32_t* ncodes) {
    const long long N = c->g.N;
    unsigned long long* keys = nullptr;
    T* vals = nullptr;
    int* slot_code = nullptr;
    int* status = nullptr;
    void* tab = nullptr;
    unsigned short* code = nullptr;
    auto release = [&](bool keep) {
        dfree(keys, c->own);
        dfree(vals, c->own);
        dfree(slot_code, c->own);
        dfree(status, c->own);
        if (!keep) {
            dfree(tab, c->own);
            dfree(code, c->own);
        }
    };
    int rc = dev_alloc(c, (void**)&keys, kCodeSlots * sizeof(unsigned long long));
    if (!rc) rc = dev_alloc(c, (void**)&vals, (size_t)kCodeSlots * 9 * sizeof(T));
    if (!rc) rc = dev_alloc(c, (void**)&slot_code, kCodeSlots * sizeof(int));
    if (!rc) rc = dev_alloc(c, (void**)&status, 4 * sizeof(int));
    if (!rc) rc = dev_alloc(c, &tab, (size_t)kMaxCodes * 12 * sizeof(T));
    if (!rc) rc = dev_alloc(c, (void**)&code, (size_t)N * sizeof(unsigned short));
    if (rc) {
        release(false);
        return rc;
    }
    cudaError_t e = cudaMemsetAsync(keys, 0, kCodeSlots * sizeof(unsigned long long), c->own);
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, 4 * sizeof(int), c->own);
    const T* ch = static_cast<const T*>(c->ch);
    const T* ce = static_cast<const T*>(c->ce);
    const T* cl = static_cast<const T*>(c->cl);
    const unsigned blocks = (unsigned)std::max<long long>(1, std::min<long long>((N + 255) / 256, 8LL * c->nsm));
    if (e == cudaSuccess) {
        k_code_insert<T><<<blocks, 256, 0, c->own>>>(ch, ce, cl, N, keys, vals, status);
        k_code_number<T><<<1, 1024, 0, c->own>>>(keys, vals, slot_code, static_cast<T*>(tab), status);
        k_code_assign<T><<<blocks, 256, 0, c->own>>>(ch, ce, cl, N, keys, slot_code, static_cast<const T*>(tab),
                                                     code, status);
        count(c, 3);
        e = cudaGetLastError();
    }
    int st[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(st, status, sizeof(st), cudaMemcpyDeviceToHost, c->own);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->own);
    if (e != cudaSuccess) {
        release(false);
        return fail(c, FIT_ERR_CUDA, "coefficient codes: %s", cudaGetErrorString(e));
    }
    const bool ok = st[0] == 0 && st[1] <= kMaxCodes && st[2] == 0;
    void* exact = nullptr;  // the table at its final size
    if (ok) {
        const size_t tb = (size_t)std::max(st[1], 1) * 12 * sizeof(T);
        int rc2 = dev_alloc(c, &exact, tb);
        if (!rc2) e = cudaMemcpyAsync(exact, tab, tb, cudaMemcpyDeviceToDevice, c->own);
        if (rc2 || e != cudaSuccess) {
            dfree(exact, c->own);
            release(false);
            return rc2 ? rc2 : fail(c, FIT_ERR_CUDA, "coefficient codes: %s", cudaGetErrorString(e));
        }
        dfree(tab, c->own);
        tab = nullptr;
    }
    release(ok);
    *ncodes = ok ? st[1] : 0;
    if (ok) {
        c->d_code = code;
        c->d_tab = exact;
        c->ncodes = st[1];
    }
    return FIT_OK;
}

}  // namespace

extern "C" {

int fit_ctx_create(const FitGridDesc* d, FitCtx** out) {
    FitCtx* c = nullptr;
    if (!d || !out) return fail(nullptr, FIT_ERR_ARG, "null argument");
    *out = nullptr;
    if (d->nx < 1 || d->ny < 1 || d->nz < 1)
        return fail(nullptr, FIT_ERR_ARG, "grid dimensions must be >= 1 (got %lld x %lld x %lld)",
                    (long long)d->nx, (long long)d->ny, (long long)d->nz);
    const long long N = d->nx * d->ny * d->nz;
    // the kernels address cells by 32-bit offsets up to N + Nx*Ny from a component's start
    if (N + d->nx * d->ny >= (1LL << 31))
        return fail(nullptr, FIT_ERR_ARG, "grid too large: N = %lld cells (limit N + Nx*Ny < 2^31)", N);
    if (d->dtype != FIT_F32 && d->dtype != FIT_F64) return fail(nullptr, FIT_ERR_ARG, "dtype must be FIT_F32 or FIT_F64");
    for (int a = 0; a < 3; ++a)
        if (d->bc_lo[a] < 0 || d->bc_lo[a] > 4 || d->bc_hi[a] < 0 || d->bc_hi[a] > 4)
            return fail(nullptr, FIT_ERR_ARG, "invalid boundary code on axis %d", a);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(nullptr, FIT_ERR_DEVICE, "no CUDA device available");
    if (d->device < 0 || d->device >= ndev) return fail(nullptr, FIT_ERR_ARG, "invalid device %d", d->device);
    c = new FitCtx();
    c->device = d->device;
    c->dtype = d->dtype;
    c->use_cond = d->use_conductivity ? 1 : 0;
    c->g.nx = (int)d->nx;
    c->g.ny = (int)d->ny;
    c->g.nz = (int)d->nz;
    c->g.N = N;
    c->g.sy = d->nx;
    c->g.sz = d->nx * d->ny;
    c->g.fx = make_fastdiv((unsigned)d->nx);
    c->g.fy = make_fastdiv((unsigned)d->ny);
    // face masks (wakis/boundaries.py:73-150)
    unsigned pec = 0, pmc = 0;
    bool any_pmc = false;
    for (int a = 0; a < 3; ++a) {
        c->bc_lo[a] = d->bc_lo[a];
        c->bc_hi[a] = d->bc_hi[a];
        if (d->bc_lo[a] == FIT_BC_PEC || d->bc_lo[a] == FIT_BC_PML) pec |= 1u << (2 * a);
        if (d->bc_hi[a] == FIT_BC_PEC || d->bc_hi[a] == FIT_BC_PML) pec |= 1u << (2 * a + 1);
        if (d->bc_lo[a] == FIT_BC_PMC) { pmc |= 1u << (2 * a); any_pmc = true; }
        if (d->bc_hi[a] == FIT_BC_PMC) { pmc |= 1u << (2 * a + 1); any_pmc = true; }
    }
    c->g.pec = pec;
    c->g.pmc = any_pmc ? (pmc | pec) : 0u;  // the PMC mask starts from the PEC face values
    // periodic edits (x, y, z) then ABC high-face edits (x, y, z)
    bool any_periodic_lo = false;
    for (int a = 0; a < 3; ++a) any_periodic_lo |= d->bc_lo[a] == FIT_BC_PERIODIC;
    if (any_periodic_lo)
        for (int a = 0; a < 3; ++a)
            if (d->bc_lo[a] == FIT_BC_PERIODIC && d->bc_hi[a] == FIT_BC_PERIODIC) c->edits[c->n_edits++] = a;
    bool any_abc = false;
    for (int a = 0; a < 3; ++a) any_abc |= d->bc_lo[a] == FIT_BC_ABC || d->bc_hi[a] == FIT_BC_ABC;
    if (any_abc)
        for (int a = 0; a < 3; ++a)
            if (d->bc_hi[a] == FIT_BC_ABC) c->edits[c->n_edits++] = a;
    c->E = d->E;
    c->H = d->H;
    c->J = d->J;
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming);
    if (e == cudaSuccess) keep_freed_blocks(c->device);
    if (e == cudaSuccess) e = cudaMallocAsync(&c->d_step, sizeof(long long), c->own);
    if (e == cudaSuccess) e = cudaMallocAsync(&c->d_err, sizeof(int), c->own);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_err, 0, sizeof(int), c->own);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device);
    if (e != cudaSuccess) {
        int rc = fail(nullptr, FIT_ERR_CUDA, "context setup failed: %s", cudaGetErrorString(e));
        fit_ctx_destroy(c);
        return rc;
    }
    const size_t fb = 3 * (size_t)N * esize(c);
    int rc = dev_alloc(c, &c->ch, fb);
    if (!rc) rc = dev_alloc(c, &c->ce, fb);
    if (!rc && c->use_cond) rc = dev_alloc(c, &c->cl, fb);
    if (rc) {
        std::string m = c->err;
        fit_ctx_destroy(c);
        return fail(nullptr, rc, "%s", m.c_str());
    }
    *out = c;
    return FIT_OK;
}

int fit_ctx_destroy(FitCtx* c) {
    if (!c) return FIT_OK;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    cudaSetDevice(c->device);
    if (c->own) cudaStreamSynchronize(c->own);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    for (int a = 0; a < 3; ++a) {
        dfree(c->dL[a], c->own);
        dfree(c->dtL0[a], c->own);
        dfree(c->tL_T[a], c->own);
        dfree(c->L_T[a], c->own);
    }
    for (void* p : {c->ch, c->ce, c->cl, c->cj, c->sg, c->E2, c->H2, (void*)c->d_mon_phases, (void*)c->d_code,
                    c->d_tab, (void*)c->d_jsig})
        dfree(p, c->own);
    for (void* p : {(void*)c->d_beam_z, (void*)c->d_beam_dtieps, (void*)c->d_vt_table, (void*)c->d_prof,
                    (void*)c->d_c1, (void*)c->d_c2, (void*)c->d_gt, (void*)c->d_stash, (void*)c->d_base, (void*)c->d_row,
                    (void*)c->d_em, (void*)c->d_ek0, (void*)c->d_ecnt, (void*)c->d_dz, (void*)c->d_acc,
                    (void*)c->d_comp, (void*)c->d_scratch, (void*)c->d_wp3d, (void*)c->d_wpx, (void*)c->d_wpy,
                    (void*)c->d_step, (void*)c->d_err})
        dfree(p, c->own);
    if (c->own) cudaStreamSynchronize(c->own);
    if (c->ev_in) cudaEventDestroy(c->ev_in);
    if (c->ev_out) cudaEventDestroy(c->ev_out);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
    return FIT_OK;
}

int fit_last_error(const FitCtx* c, char* buf, int64_t len) {
    if (!buf || len <= 0) return FIT_ERR_ARG;
    std::string m;
    if (c) {
        m = c->err;
    } else {
        std::lock_guard<std::mutex> lk(g_err_mu);
        m = g_create_error;
    }
    snprintf(buf, (size_t)len, "%s", m.c_str());
    return FIT_OK;
}

int fit_set_stream(FitCtx* c, void* stream) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    c->user = static_cast<cudaStream_t>(stream);
    return FIT_OK;
}

int fit_set_fields(FitCtx* c, void* E, void* H, void* J) {
    if (!c || !E || !H || !J) return fail(c, FIT_ERR_ARG, "null field pointer");
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    invalidate(c);
    c->E = E;
    c->H = H;
    c->J = J;
    return FIT_OK;
}

int fit_set_metrics(FitCtx* c, const double* dx, const double* dy, const double* dz, const double* tdx,
                    const double* tdy, const double* tdz) {
    if (!c || !dx || !dy || !dz || !tdx || !tdy || !tdz) return fail(c, FIT_ERR_ARG, "null metric array");
    invalidate(c);
    int rc = enter(c);
    if (rc) return rc;
    const double* L[3] = {dx, dy, dz};
    const double* T0[3] = {tdx, tdy, tdz};
    const int len[3] = {c->g.nx, c->g.ny, c->g.nz};
    bool edited[3] = {false, false, false};
    for (int e = 0; e < c->n_edits; ++e) edited[c->edits[e]] = true;
    for (int a = 0; a < 3; ++a) {
        std::vector<double> tl(T0[a], T0[a] + len[a]);
        if (edited[a]) tl[len[a] - 1] = L[a][0];  // tL[-1] = L[0] (wakis/boundaries.py:41,157)
        rc = upload(c, &c->dL[a], L[a], len[a] * sizeof(double));
        if (!rc) rc = upload(c, &c->dtL0[a], T0[a], len[a] * sizeof(double));
        if (rc) return rc;
        if (c->dtype == FIT_F64) {
            rc = upload(c, reinterpret_cast<double**>(&c->L_T[a]), L[a], len[a] * sizeof(double));
            if (!rc) rc = upload(c, reinterpret_cast<double**>(&c->tL_T[a]), tl.data(), len[a] * sizeof(double));
        } else {
            std::vector<float> lf(L[a], L[a] + len[a]), tf(tl.begin(), tl.end());
            rc = upload(c, reinterpret_cast<float**>(&c->L_T[a]), lf.data(), len[a] * sizeof(float));
            if (!rc) rc = upload(c, reinterpret_cast<float**>(&c->tL_T[a]), tf.data(), len[a] * sizeof(float));
            if (!rc) CK(cudaStreamSynchronize(c->own));  // host vectors die here
        }
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(c->own));
    c->metrics_set = true;
    return leave(c);
}

int fit_enable_explicit_j(FitCtx* c) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    if (c->explicit_ready) return FIT_OK;
    const size_t fb = 3 * (size_t)c->g.N * esize(c);
    int rc = dev_alloc(c, &c->cj, fb);
    if (!rc) rc = dev_alloc(c, &c->sg, fb);
    if (rc) return rc;
    invalidate(c);
    c->explicit_ready = true;
    c->coeffs_set = false;  // cj / sg must be filled by fit_set_coeffs
    return FIT_OK;
}

int fit_set_coeffs(FitCtx* c, double dt, const double* ieps, const double* imu, const double* sigma) {
    if (!c || !ieps || !imu || !sigma) return fail(c, FIT_ERR_ARG, "null material array");
    if (!c->metrics_set) return fail(c, FIT_ERR_STATE, "fit_set_metrics must precede fit_set_coeffs");
    int rc = enter(c);
    if (rc) return rc;
    drop_codes(c);  // the codes describe the coefficients being replaced
    CoeffArgs a{};
    for (int i = 0; i < 3; ++i) {
        a.L[i] = c->dL[i];
        a.tL[i] = c->dtL0[i];
    }
    for (int e = 0; e < c->n_edits; ++e) a.edits[e] = c->edits[e];
    a.n_edits = c->n_edits;
    a.dt = dt;
    a.use_cond = c->use_cond;
    const long long n3 = 3 * c->g.N;
    if (c->dtype == FIT_F64)
        k_build_coeffs<double><<<grid1d(n3, 256), 256, 0, c->own>>>(
            ieps, imu, sigma, (double*)c->ch, (double*)c->ce, (double*)c->cl, (double*)c->cj, (double*)c->sg, c->g, a);
    else
        k_build_coeffs<float><<<grid1d(n3, 256), 256, 0, c->own>>>(
            ieps, imu, sigma, (float*)c->ch, (float*)c->ce, (float*)c->cl, (float*)c->cj, (float*)c->sg, c->g, a);
    count(c);
    c->dt = dt;
    // beam line dt*ieps
    if (c->beam.active && !c->ieps_line.empty()) {
        std::vector<double> v(c->ieps_line.size());
        for (size_t k = 0; k < v.size(); ++k) v[k] = dt * c->ieps_line[k];
        invalidate(c);
        rc = upload(c, &c->d_beam_dtieps, v.data(), v.size() * sizeof(double));
        if (rc) return rc;
        c->beam.dtieps = c->d_beam_dtieps;
        CK(cudaStreamSynchronize(c->own));
    }
    c->coeffs_set = true;
    return leave(c);
}

int fit_zero_ghosts(FitCtx* c) {
    if (!c || !c->E || !c->H) return fail(c, FIT_ERR_STATE, "fields not set");
    int rc = enter(c);
    if (rc) return rc;
    if (c->dtype == FIT_F64)
        k_zero_ghosts<double><<<grid1d(c->g.N, 256), 256, 0, c->own>>>((double*)c->E, (double*)c->H, c->g);
    else
        k_zero_ghosts<float><<<grid1d(c->g.N, 256), 256, 0, c->own>>>((float*)c->E, (float*)c->H, c->g);
    g_launches++;
    return leave(c);
}

int fit_set_beam(FitCtx* c, int32_t active, int32_t ixs, int32_t iys, double q, double v, double sigmaz, double s0,
                 double dx_s, double dy_s, const double* z, const double* ieps_line) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    invalidate(c);
    if (!active) {
        c->beam.active = 0;
        return FIT_OK;
    }
    if (ixs < 0 || ixs >= c->g.nx || iys < 0 || iys >= c->g.ny) return fail(c, FIT_ERR_ARG, "beam cell out of range");
    if (!z || !ieps_line) return fail(c, FIT_ERR_ARG, "null beam array");
    if (!(sigmaz > 0)) return fail(c, FIT_ERR_ARG, "sigmaz must be > 0");
    int rc = enter(c);
    if (rc) return rc;
    rc = upload(c, &c->d_beam_z, z, c->g.nz * sizeof(double));
    if (rc) return rc;
    c->ieps_line.assign(ieps_line, ieps_line + c->g.nz);
    std::vector<double> dv(c->g.nz);
    for (int k = 0; k < c->g.nz; ++k) dv[k] = c->dt * ieps_line[k];
    rc = upload(c, &c->d_beam_dtieps, dv.data(), dv.size() * sizeof(double));
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->own));
    BeamArgs& b = c->beam;
    b.active = 1;
    b.ixs = ixs;
    b.iys = iys;
    b.qv = q * v;
    // numpy evaluates 2 * np.pi * sigmaz**2 as (2*pi)*(sigmaz*sigmaz)
    const double s2 = sigmaz * sigmaz;
    b.c0 = 1.0 / sqrt((2.0 * 3.141592653589793) * s2);
    b.two_s2 = 2.0 * s2;
    b.s0 = s0;
    b.dx_s = dx_s;
    b.dy_s = dy_s;
    b.z = c->d_beam_z;
    b.dtieps = c->d_beam_dtieps;
    return leave(c);
}

int fit_set_beam_vt(FitCtx* c, double vt) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    c->beam_vt = vt;
    return FIT_OK;
}

int fit_set_beam_vt_table(FitCtx* c, const double* vt, int64_t n) {
    if (!c || (!vt && n > 0) || n < 0) return fail(c, FIT_ERR_ARG, "bad vt table");
    int rc = enter(c);
    if (rc) return rc;
    invalidate(c);
    rc = upload(c, &c->d_vt_table, vt, n * sizeof(double));
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->own));
    c->vt_len = n;
    return leave(c);
}

int fit_set_plane_source(FitCtx* c, int32_t active, int32_t zs, int32_t x0, int32_t x1, int32_t y0, int32_t y1,
                         const double* prof, const double* c1, const double* c2, const double* gt, int64_t n) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    invalidate(c);
    if (!active) {
        c->plane.active = 0;
        return FIT_OK;
    }
    if (zs < 0 || zs >= c->g.nz || x0 < 0 || x1 > c->g.nx || x0 >= x1 || y0 < 0 || y1 > c->g.ny || y0 >= y1)
        return fail(c, FIT_ERR_ARG, "plane source region out of range");
    if (!c1 || !c2 || !gt || n <= 0) return fail(c, FIT_ERR_ARG, "bad plane source tables");
    int rc = enter(c);
    if (rc) return rc;
    const size_t np = (size_t)(x1 - x0) * (y1 - y0);
    if (prof) {
        rc = upload(c, &c->d_prof, prof, np * sizeof(double));
    } else {
        dfree(c->d_prof, c->own);
        c->d_prof = nullptr;
    }
    if (!rc) rc = upload(c, &c->d_c1, c1, n * sizeof(double));
    if (!rc) rc = upload(c, &c->d_c2, c2, n * sizeof(double));
    if (!rc) rc = upload(c, &c->d_gt, gt, n * sizeof(double));
    if (!rc) rc = dev_alloc(c, (void**)&c->d_stash, np * sizeof(double));
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->own));
    PlaneArgs& p = c->plane;
    p.stash = c->d_stash;
    p.active = 1;
    p.zs = zs;
    p.x0 = x0;
    p.x1 = x1;
    p.y0 = y0;
    p.y1 = y1;
    p.prof = c->d_prof;
    p.c1 = c->d_c1;
    p.c2 = c->d_c2;
    p.gt = c->d_gt;
    p.len = n;
    return leave(c);
}

int fit_set_abc(FitCtx* c, int32_t lo_axes) {
    if (!c || lo_axes < 0 || lo_axes > 7) return fail(c, FIT_ERR_ARG, "bad abc axes");
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    const int len[3] = {c->g.nx, c->g.ny, c->g.nz};
    for (int a = 0; a < 3; ++a)
        if ((lo_axes >> a) & 1)
            if (len[a] < 2) return fail(c, FIT_ERR_ARG, "ABC on axis %d needs at least 2 cells", a);
    if (lo_axes != c->abc_axes) invalidate(c);
    c->abc_axes = lo_axes;
    return FIT_OK;
}

int fit_set_wake_taps(FitCtx* c, int32_t nlines, const int32_t* lx, const int32_t* ly, int32_t kskip, int32_t ns,
                      int64_t nsteps, const int64_t* row_ptr, const int32_t* ent_m, const int32_t* ent_k0,
                      const int32_t* ent_cnt, int32_t nz_tap, const double* dz) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    invalidate(c);
    if (nlines <= 0) {
        c->tap.nlines = 0;
        return FIT_OK;
    }
    if (!lx || !ly || !row_ptr || ns <= 0 || nsteps <= 0 || nz_tap <= 0 || !dz)
        return fail(c, FIT_ERR_ARG, "bad wake tap arguments");
    const long long ne = row_ptr[nsteps];
    if (ne > 0 && (!ent_m || !ent_k0 || !ent_cnt)) return fail(c, FIT_ERR_ARG, "null tap entries");
    std::vector<long long> base(nlines);
    for (int l = 0; l < nlines; ++l) {
        if (lx[l] < 0 || lx[l] >= c->g.nx || ly[l] < 0 || ly[l] >= c->g.ny)
            return fail(c, FIT_ERR_ARG, "tap line %d outside the grid", l);
        base[l] = lx[l] + c->g.sy * ly[l] + c->g.sz * (long long)kskip;
    }
    for (long long e = 0; e < ne; ++e) {
        if (ent_m[e] < 0 || ent_m[e] >= ns || ent_k0[e] < 0 || ent_cnt[e] < 1 || ent_k0[e] + ent_cnt[e] > nz_tap ||
            kskip + ent_k0[e] + ent_cnt[e] > c->g.nz)
            return fail(c, FIT_ERR_ARG, "tap entry %lld out of range", e);
    }
    int rc = enter(c);
    if (rc) return rc;
    rc = upload(c, &c->d_base, base.data(), nlines * sizeof(long long));
    if (!rc) rc = upload(c, &c->d_row, row_ptr, (nsteps + 1) * sizeof(long long));
    if (!rc) rc = upload(c, &c->d_em, ent_m, ne * sizeof(int));
    if (!rc) rc = upload(c, &c->d_ek0, ent_k0, ne * sizeof(int));
    if (!rc) rc = upload(c, &c->d_ecnt, ent_cnt, ne * sizeof(int));
    if (!rc) rc = upload(c, &c->d_dz, dz, nz_tap * sizeof(double));
    const size_t ab = (size_t)nlines * ns * sizeof(double);
    if (!rc) rc = dev_alloc(c, (void**)&c->d_acc, ab);
    if (!rc) rc = dev_alloc(c, (void**)&c->d_comp, ab);
    if (!rc) rc = dev_alloc(c, (void**)&c->d_wp3d, ab);
    if (!rc) rc = dev_alloc(c, (void**)&c->d_wpx, ns * sizeof(double));
    if (!rc) rc = dev_alloc(c, (void**)&c->d_wpy, ns * sizeof(double));
    if (!rc) rc = dev_alloc(c, (void**)&c->d_scratch, 4 * (size_t)ns * sizeof(double));
    if (rc) return rc;
    CK(cudaMemsetAsync(c->d_acc, 0, ab, c->own));
    CK(cudaMemsetAsync(c->d_comp, 0, ab, c->own));
    CK(cudaStreamSynchronize(c->own));
    TapArgs& t = c->tap;
    t.nlines = nlines;
    t.base = c->d_base;
    t.ns = ns;
    t.nsteps = nsteps;
    t.row_ptr = c->d_row;
    t.ent_m = c->d_em;
    t.ent_k0 = c->d_ek0;
    t.ent_cnt = c->d_ecnt;
    t.dz = c->d_dz;
    t.acc = c->d_acc;
    t.comp = c->d_comp;
    return leave(c);
}

int fit_reset_wake(FitCtx* c) {
    if (!c) return FIT_ERR_ARG;
    if (c->tap.nlines <= 0) return FIT_OK;
    int rc = enter(c);
    if (rc) return rc;
    const size_t ab = (size_t)c->tap.nlines * c->tap.ns * sizeof(double);
    CK(cudaMemsetAsync(c->d_acc, 0, ab, c->own));
    CK(cudaMemsetAsync(c->d_comp, 0, ab, c->own));
    return leave(c);
}

int fit_read_wake(FitCtx* c, double* out) {
    if (!c || !out) return FIT_ERR_ARG;
    if (c->tap.nlines <= 0) return fail(c, FIT_ERR_STATE, "no wake taps set");
    int rc = enter(c);
    if (rc) return rc;
    const size_t n = (size_t)c->tap.nlines * c->tap.ns;
    std::vector<double> a(n), b(n);
    CK(cudaMemcpyAsync(a.data(), c->d_acc, n * sizeof(double), cudaMemcpyDeviceToHost, c->own));
    CK(cudaMemcpyAsync(b.data(), c->d_comp, n * sizeof(double), cudaMemcpyDeviceToHost, c->own));
    CK(cudaStreamSynchronize(c->own));
    for (size_t i = 0; i < n; ++i) out[i] = a[i] + b[i];
    return leave(c);
}

int fit_step(FitCtx* c, int64_t n, int32_t j_mode) {
    int rc = check_ready(c);
    if (rc) return rc;
    const bool beam_off = (j_mode & FIT_STEP_NO_BEAM) != 0;
    j_mode &= ~FIT_STEP_NO_BEAM;
    int mode;
    if (j_mode == FIT_J_EXPLICIT) {
        if (!c->explicit_ready) return fail(c, FIT_ERR_STATE, "explicit-J storage not enabled");
        mode = 2;
    } else if (j_mode == FIT_J_ELIDED) {
        mode = c->use_cond ? 1 : 0;
    } else {
        return fail(c, FIT_ERR_ARG, "bad j_mode %d", j_mode);
    }
    if (c->beam.active && !c->beam.dtieps) return fail(c, FIT_ERR_STATE, "beam set before coefficients");
    rc = enter(c);
    if (rc) return rc;
    const int saved = c->beam.active;
    if (beam_off) c->beam.active = 0;
    launch_step(c, n, mode, false);
    c->beam.active = saved;
    return leave(c);
}

int fit_run(FitCtx* c, int64_t n0, int64_t nsteps) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (nsteps < 0) return fail(c, FIT_ERR_ARG, "nsteps < 0");
    if (nsteps == 0) return FIT_OK;
    if (c->beam.active && (c->vt_len < n0 + nsteps))
        return fail(c, FIT_ERR_STATE, "beam vt table shorter than the run (%lld < %lld)", c->vt_len,
                    (long long)(n0 + nsteps));
    const int mode = c->use_cond ? 1 : 0;
    rc = enter(c);
    if (rc) return rc;
    static thread_local long long host_n0;
    host_n0 = n0;
    CK(cudaMemcpyAsync(c->d_step, &host_n0, sizeof(long long), cudaMemcpyHostToDevice, c->own));
    CK(cudaStreamSynchronize(c->own));
    const long long chunk = 64;
    if (fused_ok(c, mode)) {
        // pairs of fused steps leave the state in the caller's buffers; an odd count
        // takes its first step with the in-place two-pass kernels
        const StepArgs st = device_step_args(c);
        long long done = 0;
        if (nsteps % 2) {
            launch_step(c, 0, mode, true);
            done = 1;
        }
        if (nsteps - done >= chunk && (!c->graph || c->graph_chunk != chunk || !c->graph_fused)) {
            invalidate(c);
            cudaGraph_t gr;
            CK(cudaStreamBeginCapture(c->own, cudaStreamCaptureModeThreadLocal));
            c->capturing = true;
            for (long long s = 0; s < chunk; s += 2) {
                launch_fused_step(c, mode, true, st, 0);
                launch_fused_step(c, mode, false, st, 0);
            }
            c->capturing = false;
            cudaError_t e = cudaStreamEndCapture(c->own, &gr);
            if (e != cudaSuccess) return fail(c, FIT_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&c->graph, gr, 0);
            cudaGraphDestroy(gr);
            if (e != cudaSuccess) return fail(c, FIT_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
            c->graph_chunk = chunk;
            c->graph_fused = true;
        }
        while (nsteps - done >= chunk) {
            CK(cudaGraphLaunch(c->graph, c->own));
            g_launches += chunk * (2 + (c->mon.nf > 0));
            done += chunk;
        }
        for (; done < nsteps; done += 2) {
            launch_fused_step(c, mode, true, st, 0);
            launch_fused_step(c, mode, false, st, 0);
        }
        return leave(c);
    }
    if (nsteps >= chunk) {
        if (!c->graph || c->graph_chunk != chunk || c->graph_fused) {
            if (c->graph) {
                cudaGraphExecDestroy(c->graph);
                c->graph = nullptr;
            }
            cudaGraph_t gr;
            CK(cudaStreamBeginCapture(c->own, cudaStreamCaptureModeThreadLocal));
            c->capturing = true;
            for (long long s = 0; s < chunk; ++s) launch_step(c, 0, mode, true);
            c->capturing = false;
            cudaError_t e = cudaStreamEndCapture(c->own, &gr);
            if (e != cudaSuccess) return fail(c, FIT_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&c->graph, gr, 0);
            cudaGraphDestroy(gr);
            if (e != cudaSuccess) return fail(c, FIT_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
            c->graph_chunk = chunk;
            c->graph_fused = false;
        }
    }
    long long done = 0;
    while (nsteps - done >= chunk) {
        CK(cudaGraphLaunch(c->graph, c->own));
        g_launches += chunk * launches_per_step(c);
        done += chunk;
    }
    for (; done < nsteps; ++done) launch_step(c, 0, mode, true);
    return leave(c);
}

int fit_materialize_J(FitCtx* c, const double* sigma, int32_t flags) {
    if (!c) return FIT_ERR_ARG;
    const bool do_sig = (flags & 1) && c->use_cond;
    const bool do_beam = (flags & 2) && c->beam.active;
    if (do_sig && !sigma) return fail(c, FIT_ERR_ARG, "sigma required");
    int rc = enter(c);
    if (rc) return rc;
    const long long n3 = 3 * c->g.N;
    if (c->dtype == FIT_F64) {
        if (do_sig) {
            k_materialize_J<double><<<grid1d(n3, 256), 256, 0, c->own>>>((const double*)c->E, (double*)c->J, sigma, c->g, 1);
            count(c);
        }
        if (do_beam) {
            k_beam_line<double><<<grid1d(c->g.nz, 128), 128, 0, c->own>>>((double*)c->J, c->g, c->beam, c->beam_vt);
            count(c);
        }
    } else {
        if (do_sig) {
            k_materialize_J<float><<<grid1d(n3, 256), 256, 0, c->own>>>((const float*)c->E, (float*)c->J, sigma, c->g, 1);
            count(c);
        }
        if (do_beam) {
            k_beam_line<float><<<grid1d(c->g.nz, 128), 128, 0, c->own>>>((float*)c->J, c->g, c->beam, c->beam_vt);
            count(c);
        }
    }
    return leave(c);
}

int fit_wake_finalize(FitCtx* c, double qscale, double ds, double dxf, double dyf, double* wp3d, double* wpx,
                      double* wpy) {
    if (!c || !wp3d) return FIT_ERR_ARG;
    if (c->tap.nlines <= 0) return fail(c, FIT_ERR_STATE, "no wake taps set");
    int rc = enter(c);
    if (rc) return rc;
    const int nl = c->tap.nlines, ns = c->tap.ns;
    k_wake_finalize<<<1, 1024, 0, c->own>>>(c->d_acc, c->d_comp, nl, ns, qscale, ds, dxf, dyf, c->d_wp3d, c->d_wpx,
                                            c->d_wpy, c->d_scratch, nl == 9 ? 3 : 0);
    g_launches++;
    CK(cudaMemcpyAsync(wp3d, c->d_wp3d, (size_t)nl * ns * sizeof(double), cudaMemcpyDeviceToHost, c->own));
    if (nl == 9 && wpx && wpy) {
        CK(cudaMemcpyAsync(wpx, c->d_wpx, ns * sizeof(double), cudaMemcpyDeviceToHost, c->own));
        CK(cudaMemcpyAsync(wpy, c->d_wpy, ns * sizeof(double), cudaMemcpyDeviceToHost, c->own));
    }
    CK(cudaStreamSynchronize(c->own));
    return leave(c);
}

// side of a square of nlines = side*side lines with an odd side >= 3 (a transverse wake
// exists), else 0
static int square_side(int nlines) {
    for (int q = 3; q * q <= nlines; q += 2)
        if (q * q == nlines) return q;
    return 0;
}

int fit_wake_history(const double* ezt, int32_t nlines, int64_t nt, int32_t nz, const int32_t* it, int32_t ns,
                     const double* dz, double qscale, double ds, double dxf, double dyf, double* wp3d, double* wpx,
                     double* wpy) {
    if (!ezt || !it || !dz || !wp3d || nlines <= 0 || nt <= 0 || nz <= 0 || ns <= 0 || nt > INT32_MAX)
        return fail(nullptr, FIT_ERR_ARG, "bad fit_wake_history arguments");
    const size_t n_ezt = (size_t)nlines * nz * nt, n_it = (size_t)nz * ns;
    double *d_ezt = nullptr, *d_dz = nullptr, *d_wp = nullptr, *d_wpx = nullptr, *d_wpy = nullptr,
           *d_scr = nullptr;
    int* d_it = nullptr;
    cudaStream_t s = nullptr;
    auto cleanup = [&]() {
        if (s) {
            dfree(d_ezt, s);
            dfree(d_dz, s);
            dfree(d_wp, s);
            dfree(d_wpx, s);
            dfree(d_wpy, s);
            dfree(d_scr, s);
            dfree(d_it, s);
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    };
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) keep_freed_blocks(dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_ezt, n_ezt * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_it, n_it * sizeof(int), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_dz, (size_t)nz * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_wp, (size_t)nlines * ns * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_wpx, (size_t)ns * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_wpy, (size_t)ns * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_scr, 4 * (size_t)ns * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_ezt, ezt, n_ezt * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_it, it, n_it * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_dz, dz, (size_t)nz * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        cleanup();
        return fail(nullptr, FIT_ERR_CUDA, "fit_wake_history setup failed: %s", cudaGetErrorString(e));
    }
    k_wake_history<<<(unsigned)((ns + 127) / 128), 128, 0, s>>>(d_ezt, nlines, nt, nz, d_it, ns, d_dz, qscale, d_wp);
    const int side = square_side(nlines);
    k_wake_finalize<<<1, 1024, 0, s>>>(nullptr, nullptr, nlines, ns, qscale, ds, dxf, dyf, d_wp, d_wpx, d_wpy,
                                       d_scr, side);
    g_launches += 2;
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(wp3d, d_wp, (size_t)nlines * ns * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && side >= 3 && wpx && wpy) {
        e = cudaMemcpyAsync(wpx, d_wpx, (size_t)ns * sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(wpy, d_wpy, (size_t)ns * sizeof(double), cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cleanup();
    if (e != cudaSuccess) return fail(nullptr, FIT_ERR_CUDA, "fit_wake_history failed: %s", cudaGetErrorString(e));
    return FIT_OK;
}

int fit_dft(const double* x, int32_t nsig, int64_t len, int64_t n, int64_t b0, int32_t nb, double* out) {
    if (!x || !out || nsig <= 0 || len <= 0 || n <= 0 || nb <= 0 || b0 < 0)
        return fail(nullptr, FIT_ERR_ARG, "bad fit_dft arguments");
    if (nsig > kDftMaxSignals)
        return fail(nullptr, FIT_ERR_ARG, "fit_dft: nsig = %d exceeds %d signals per call", nsig, kDftMaxSignals);
    const int nsplit = (int)std::max<long long>(1, std::min<long long>(32, len / 2048));
    double* dx = nullptr;
    double2* part = nullptr;
    double2* dout = nullptr;
    cudaStream_t s = nullptr;
    auto cleanup = [&]() {
        if (s) {
            dfree(dx, s);
            dfree(part, s);
            dfree(dout, s);
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    };
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) keep_freed_blocks(dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocAsync(&dx, (size_t)nsig * len * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&part, (size_t)nsig * nsplit * nb * sizeof(double2), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&dout, (size_t)nsig * nb * sizeof(double2), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, (size_t)nsig * len * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        cleanup();
        return fail(nullptr, FIT_ERR_CUDA, "fit_dft setup failed: %s", cudaGetErrorString(e));
    }
    dim3 grid((unsigned)nb, (unsigned)nsig, (unsigned)nsplit);
    k_dft_partial<<<grid, 256, 0, s>>>(dx, nsig, len, n, b0, nb, nsplit, part);
    k_dft_reduce<<<grid1d((long long)nsig * nb, 256), 256, 0, s>>>(part, nsig, nb, nsplit, dout);
    g_launches += 2;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, (size_t)nsig * nb * sizeof(double2), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cleanup();
    if (e != cudaSuccess) return fail(nullptr, FIT_ERR_CUDA, "fit_dft failed: %s", cudaGetErrorString(e));
    return FIT_OK;
}

int fit_time_kernels(FitCtx* c, int32_t reps, double* ms_out) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (reps < 1 || !ms_out) return fail(c, FIT_ERR_ARG, "bad timing arguments");
    rc = enter(c);
    if (rc) return rc;
    cudaEvent_t e0, e1, e2;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventCreate(&e2));
    const int mode = c->use_cond ? 1 : 0;
    StepArgs st{};
    st.vt = c->beam_vt;
    const int vec = pick_vec(c);
    auto h = [&]() {
        if (c->dtype == FIT_F64) {
            if (vec == 2) launch_h<double, 2>(c); else launch_h<double, 1>(c);
        } else {
            if (vec == 4) launch_h<float, 4>(c); else if (vec == 2) launch_h<float, 2>(c); else launch_h<float, 1>(c);
        }
    };
    auto e = [&]() {
        if (c->dtype == FIT_F64) {
            if (vec == 2) launch_e<double, 2>(c, mode, st); else launch_e<double, 1>(c, mode, st);
        } else {
            if (vec == 4) launch_e<float, 4>(c, mode, st);
            else if (vec == 2) launch_e<float, 2>(c, mode, st);
            else launch_e<float, 1>(c, mode, st);
        }
    };
    CK(cudaEventRecord(e0, c->own));
    for (int r = 0; r < reps; ++r) h();
    CK(cudaEventRecord(e1, c->own));
    for (int r = 0; r < reps; ++r) e();
    CK(cudaEventRecord(e2, c->own));
    CK(cudaEventSynchronize(e2));
    float a = 0.f, b = 0.f;
    CK(cudaEventElapsedTime(&a, e0, e1));
    CK(cudaEventElapsedTime(&b, e1, e2));
    ms_out[0] = a / reps;
    ms_out[1] = b / reps;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    return leave(c);
}

int fit_check_error(FitCtx* c) {
    if (!c) return FIT_ERR_ARG;
    int rc = enter(c);
    if (rc) return rc;
    int h = 0;
    CK(cudaMemcpyAsync(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->own));
    CK(cudaStreamSynchronize(c->own));
    rc = leave(c);
    if (rc) return rc;
    if (h != 0) {
        int z = 0;
        cudaMemcpy(c->d_err, &z, sizeof(int), cudaMemcpyHostToDevice);
        return fail(c, h, "a kernel gave up waiting for its bulk copies (error %d)", h);
    }
    return FIT_OK;
}

int fit_set_wait_limit(FitCtx* c, int64_t polls) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    if (polls < 0) return fail(c, FIT_ERR_ARG, "polls must be >= 0 (0: give up at once)");
    invalidate(c);
    c->wait_limit = polls;
    return FIT_OK;
}

int fit_set_kernel_variant(FitCtx* c, int32_t variant) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    if (variant < 0 || variant > 2) return fail(c, FIT_ERR_ARG, "variant must be 0 (direct), 1 (staged) or 2 (fused)");
    invalidate(c);
    c->staged = variant == 1;
    c->fused = variant == 2;
    if (c->fused && !c->E2) {
        const size_t fb = 3 * (size_t)c->g.N * esize(c);
        int rc = dev_alloc(c, &c->E2, fb);
        if (!rc) rc = dev_alloc(c, &c->H2, fb);
        if (rc) {
            c->fused = false;
            return rc;
        }
        fused_default_shape(c);
    }
    return FIT_OK;
}

int fit_set_coeff_codes(FitCtx* c, int32_t enable, int32_t* ncodes) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    int32_t dummy = 0;
    if (!ncodes) ncodes = &dummy;
    *ncodes = 0;
    if (!enable) {
        drop_codes(c);
        return FIT_OK;
    }
    if (!c->coeffs_set || !c->ch || !c->ce) return fail(c, FIT_ERR_STATE, "fit_set_coeffs must precede the codes");
    if (c->d_code) {
        *ncodes = c->ncodes;
        return FIT_OK;
    }
    int rc = enter(c);
    if (rc) return rc;
    invalidate(c);
    rc = c->dtype == FIT_F64 ? build_codes_t<double>(c, ncodes) : build_codes_t<float>(c, ncodes);
    if (rc) return rc;
    return leave(c);
}

int fit_set_fused_shape(FitCtx* c, int32_t vec, int32_t rows, int32_t zseg, int32_t ctas) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    const bool vec_ok = (vec == 2 && c->g.nx % 2 == 0) || (vec == 4 && c->dtype == FIT_F32 && c->g.nx % 4 == 0);
    if (ctas == 0) ctas = rows == 8 ? 2 : 3;
    const bool ctas_ok = (rows == 8 && ctas == 2) || (rows == 4 && (ctas == 3 || ctas == 4));
    if (!vec_ok || !ctas_ok || zseg < 1 || zseg > c->g.nz)
        return fail(c, FIT_ERR_ARG, "bad fused tile shape (vec %d, rows %d, z ranges %d, CTAs/SM %d)", vec, rows, zseg,
                    ctas);
    invalidate(c);
    c->fused_vec = vec;
    c->fused_rows = rows;
    c->fused_zseg = zseg;
    c->fused_ctas = ctas;
    return FIT_OK;
}

int fit_set_fused_staging(FitCtx* c, int32_t staging, int32_t l2_ahead) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    if (staging < 0 || staging > 2) return fail(c, FIT_ERR_ARG, "staging must be 0 (loads), 1 or 2 (TMA rings)");
    if (l2_ahead < 0 || l2_ahead > 16) return fail(c, FIT_ERR_ARG, "l2_ahead must be in [0, 16]");
    if (staging != 0) {
        if (!c->fused || !c->E2) return fail(c, FIT_ERR_STATE, "the fused step is not enabled for this context");
        if (!tma_grid_ok(c))
            return fail(c, FIT_ERR_ARG, "TMA staging needs coded coefficients, Nx %% 8 == 0 and (FP32) 4-wide vectors");
        if (!tma_maps_ok(c, staging, c->fused_rows))
            return fail(c, FIT_ERR_ARG, "the TMA tensor maps of this grid cannot be encoded");
    }
    invalidate(c);
    c->fused_staging = staging;
    c->tma_prefetch = l2_ahead;
    return FIT_OK;
}

int fit_set_monitor(FitCtx* c, int32_t nf, const double* phases, int64_t n0, int64_t nsteps, void* acc,
                    int32_t single) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    invalidate(c);
    if (nf <= 0) {
        c->mon = MonitorArgs{};
        return FIT_OK;
    }
    if (!phases || !acc || nsteps <= 0 || n0 < 0) return fail(c, FIT_ERR_ARG, "bad field monitor arguments");
    int rc = enter(c);
    if (rc) return rc;
    rc = upload(c, &c->d_mon_phases, phases, (size_t)nsteps * nf * sizeof(double2));
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->own));
    c->mon.nf = nf;
    c->mon.single = single != 0;
    c->mon.phases = c->d_mon_phases;
    c->mon.n0 = n0;
    c->mon.nsteps = nsteps;
    c->mon.acc = static_cast<double2*>(acc);
    return leave(c);
}

int fit_set_ez_record(FitCtx* c, void* hist, int32_t nlines, const int32_t* lx, const int32_t* ly, int64_t n0,
                      int64_t nsteps) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    invalidate(c);
    if (nlines <= 0) {
        c->rec = RecordArgs{};
        return FIT_OK;
    }
    if (nlines > 9 || !hist || !lx || !ly || n0 < 0 || nsteps <= 0) return fail(c, FIT_ERR_ARG, "bad Ez record arguments");
    RecordArgs r{};
    for (int l = 0; l < nlines; ++l) {
        if (lx[l] < 0 || lx[l] >= c->g.nx || ly[l] < 0 || ly[l] >= c->g.ny)
            return fail(c, FIT_ERR_ARG, "Ez record line %d outside the grid", l);
        r.base[l] = (long long)lx[l] + c->g.sy * ly[l];
    }
    r.hist = hist;
    r.nlines = nlines;
    r.n0 = n0;
    r.nsteps = nsteps;
    c->rec = r;
    return FIT_OK;
}

int fit_set_jz_record(FitCtx* c, void* hist, int32_t nlines, const int32_t* lx, const int32_t* ly, int64_t n0,
                      int64_t nsteps, const double* sigma_lines) {
    if (!c) return FIT_ERR_ARG;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is running in a pool");
    invalidate(c);
    if (nlines <= 0) {
        c->jrec = JRecordArgs{};
        return FIT_OK;
    }
    if (nlines > 9 || !hist || !lx || !ly || !sigma_lines || n0 < 0 || nsteps <= 0)
        return fail(c, FIT_ERR_ARG, "bad Jz record arguments");
    JRecordArgs r{};
    for (int l = 0; l < nlines; ++l) {
        if (lx[l] < 0 || lx[l] >= c->g.nx || ly[l] < 0 || ly[l] >= c->g.ny)
            return fail(c, FIT_ERR_ARG, "Jz record line %d outside the grid", l);
        r.base[l] = (long long)lx[l] + c->g.sy * ly[l];
    }
    int rc = enter(c);
    if (rc) return rc;
    rc = upload(c, &c->d_jsig, sigma_lines, (size_t)nlines * c->g.nz * sizeof(double));
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->own));
    r.hist = hist;
    r.nlines = nlines;
    r.n0 = n0;
    r.nsteps = nsteps;
    r.sig = c->d_jsig;
    c->jrec = r;
    return leave(c);
}

int fit_time_fused(FitCtx* c, int32_t reps, double* ms_out) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (reps < 1 || !ms_out) return fail(c, FIT_ERR_ARG, "bad timing arguments");
    const int mode = c->use_cond ? 1 : 0;
    if (!fused_ok(c, mode)) return fail(c, FIT_ERR_STATE, "the fused step is not enabled for this context");
    rc = enter(c);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    StepArgs st{};
    BeamArgs nobeam = c->beam;
    nobeam.active = 0;
    launch_fused(c, mode, st, true, nobeam);  // warm-up
    CK(cudaEventRecord(e0, c->own));
    for (int r = 0; r < reps; ++r) launch_fused(c, mode, st, true, nobeam);
    CK(cudaEventRecord(e1, c->own));
    CK(cudaEventSynchronize(e1));
    float a = 0.f;
    CK(cudaEventElapsedTime(&a, e0, e1));
    ms_out[0] = a / reps;
    // the two-pass step, in place on copies of the fields in the second buffers
    const size_t fb = 3 * (size_t)c->g.N * esize(c);
    CK(cudaMemcpyAsync(c->E2, c->E, fb, cudaMemcpyDeviceToDevice, c->own));
    CK(cudaMemcpyAsync(c->H2, c->H, fb, cudaMemcpyDeviceToDevice, c->own));
    std::swap(c->E, c->E2);
    std::swap(c->H, c->H2);
    const int saved = c->beam.active;
    c->beam.active = 0;
    const int vec = pick_vec(c);
    auto pass_pair = [&]() {
        if (c->dtype == FIT_F64) {
            launch_h<double, 2>(c);
            launch_e<double, 2>(c, mode, st);
        } else if (vec == 4) {
            launch_h<float, 4>(c);
            launch_e<float, 4>(c, mode, st);
        } else {
            launch_h<float, 2>(c);
            launch_e<float, 2>(c, mode, st);
        }
    };
    pass_pair();  // warm-up
    cudaEventRecord(e0, c->own);
    for (int r = 0; r < reps; ++r) pass_pair();
    cudaEventRecord(e1, c->own);
    cudaError_t err = cudaEventSynchronize(e1);
    std::swap(c->E, c->E2);
    std::swap(c->H, c->H2);
    c->beam.active = saved;
    if (err != cudaSuccess) return fail(c, FIT_ERR_CUDA, "fit_time_fused: %s", cudaGetErrorString(err));
    CK(cudaEventElapsedTime(&a, e0, e1));
    ms_out[1] = a / reps;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return leave(c);
}

int fit_version(char* buf, int64_t len) {
    if (!buf || len <= 0) return FIT_ERR_ARG;
    snprintf(buf, (size_t)len, "wakis_gb300 fit 0.1 sm_103a cuda %d", CUDART_VERSION);
    return FIT_OK;
}

int64_t fit_launch_count(void) { return g_launches.load(); }

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Allocation-free DFT.  Some callers cannot allocate device memory at the moment they need
// an impedance spectrum: a serving process that has handed all of HBM to a pool it manages
// itself (field storage for many concurrent solves), or a caller that must not pay the
// device-wide synchronisation that cudaMalloc / cudaFree imply while solver kernels are
// running on other streams.  fit_dft_noalloc takes device inputs and outputs from the
// caller and keeps its partial sums in a fixed file-scope device array instead of
// allocating.  That array (kDftScratchEntries double2 = 4 MiB) is resident on every GPU
// that loads this library until the process exits; every call on a device shares it.
namespace {

constexpr long long kDftScratchEntries = 1LL << 18;  // double2 partial sums (4 MiB)
__device__ __align__(256) double2 g_dft_scratch[kDftScratchEntries];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double2* g_scratch_ptr[kMaxDevices] = {};

// device address of g_dft_scratch on the current device, looked up once per device
// (host code only sees a host-side stand-in for the symbol)
int scratch_address(int dev, double2** out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(nullptr, FIT_ERR_DEVICE, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_dft_scratch);
        if (e != cudaSuccess)
            return fail(nullptr, FIT_ERR_CUDA, "cudaGetSymbolAddress(g_dft_scratch) failed: %s", cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<double2*>(p);
    }
    *out = g_scratch_ptr[dev];
    return FIT_OK;
}

}  // namespace

// a device (or managed) allocation visible from device `dev`; the query allocates nothing
static bool on_device(const void* p, int dev) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // clear the sticky-free error of the query
        return false;
    }
    return (a.type == cudaMemoryTypeDevice && a.device == dev) || a.type == cudaMemoryTypeManaged;
}

extern "C" int fit_dft_noalloc(const double* x, int32_t nsig, int64_t len, int64_t n, int64_t b0, int32_t nb,
                               double* out, void* stream) {
    if (!x || !out || nsig <= 0 || len <= 0 || n <= 0 || nb <= 0 || b0 < 0)
        return fail(nullptr, FIT_ERR_ARG, "bad fit_dft_noalloc arguments");
    if (nsig > kDftMaxSignals)
        return fail(nullptr, FIT_ERR_ARG, "fit_dft_noalloc: nsig = %d exceeds %d signals per call", nsig,
                    kDftMaxSignals);
    const long long per_split = (long long)nsig * nb;
    if (per_split > kDftScratchEntries)
        return fail(nullptr, FIT_ERR_ARG,
                    "fit_dft_noalloc: nsig*nb = %lld exceeds the fixed scratch of %lld partial sums", per_split,
                    kDftScratchEntries);
    int nsplit = (int)std::max<long long>(1, std::min<long long>(32, len / 2048));
    while ((long long)nsplit * per_split > kDftScratchEntries && nsplit > 1) --nsplit;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(nullptr, FIT_ERR_CUDA, "cudaGetDevice failed: %s", cudaGetErrorString(e));
    if (!on_device(x, dev) || !on_device(out, dev))
        return fail(nullptr, FIT_ERR_ARG, "fit_dft_noalloc: x and out must be device memory of the current device %d",
                    dev);
    double2* part = nullptr;
    int rc = scratch_address(dev, &part);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // every partial read by the reduction is written by this call's first kernel, so the
    // scratch needs no clearing; calls that overlap on the GPU share it and race
    dim3 grid((unsigned)nb, (unsigned)nsig, (unsigned)nsplit);
    k_dft_partial<<<grid, 256, 0, s>>>(x, nsig, len, n, b0, nb, nsplit, part);
    k_dft_reduce<<<grid1d((long long)nsig * nb, 256), 256, 0, s>>>(part, nsig, nb, nsplit,
                                                                  reinterpret_cast<double2*>(out));
    g_launches += 2;
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(nullptr, FIT_ERR_CUDA, "fit_dft_noalloc launch failed: %s", cudaGetErrorString(e));
    return FIT_OK;
}

// serving pool (continuous batching of FP32 wake solves)
#include "fit_pool.cuh"

// ---------------------------------------------------------------------------------------
// Host-driven field monitor update (FieldMonitor.update): acc += E * phase, stream-ordered.
extern "C" int fit_monitor_update(const void* E, int32_t dtype, int64_t N, int32_t nf, const double* phase, void* acc,
                                  int32_t single, void* stream) {
    if (!E || !phase || !acc || N <= 0 || nf <= 0 || (dtype != FIT_F32 && dtype != FIT_F64))
        return fail(nullptr, FIT_ERR_ARG, "bad fit_monitor_update arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) keep_freed_blocks(dev);
    double2* dph = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync(&dph, nf * sizeof(double2), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dph, phase, nf * sizeof(double2), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail(nullptr, FIT_ERR_CUDA, "fit_monitor_update: %s", cudaGetErrorString(e));
    MonitorArgs m{};
    m.nf = nf;
    m.single = single != 0;
    m.phases = dph;
    m.acc = static_cast<double2*>(acc);
    const unsigned grid = (unsigned)std::min<long long>(grid1d(3 * N, 256), 4096);
    if (dtype == FIT_F64)
        k_monitor<double><<<grid, 256, 0, st>>>(static_cast<const double*>(E), N, m, nullptr, -1);
    else
        k_monitor<float><<<grid, 256, 0, st>>>(static_cast<const float*>(E), N, m, nullptr, -1);
    g_launches++;
    e = cudaGetLastError();
    cudaFreeAsync(dph, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host phase array is read before returning
    if (e != cudaSuccess) return fail(nullptr, FIT_ERR_CUDA, "fit_monitor_update: %s", cudaGetErrorString(e));
    return FIT_OK;
}
