// fit_pool.cuh -- serving pool: continuous batching of FP32 wake solves on one GPU.
// Part of the fit_capi.cu translation unit (included at its end; uses its helpers).
//
// Threads: the caller's threads call reserve / release / submit / poll / stats; one
// driver thread per pool launches chunks and retires solves.  Shared state is guarded by
// FitPool::mu.  The driver is the only thread that issues work on the pool stream.
//
// Chunks: chunk k reads device table k&1 (rows = member contexts, ordered by vector
// width class) and replays the graph of that table and of the classes present (built
// on first use: chunk_steps x [taps + counters, the H pass of each class present, the
// E pass of each class present]).  Up to two chunks are in flight; before the table of
// chunk k+1 is staged into pinned buffer (k+1)&1 the driver has waited for chunk k-1,
// the last user of that buffer and of its device table.  Which contexts a chunk
// finishes is known on the host when it is launched (every member takes min(chunk,
// remaining) steps), so no device state is read back between chunks.
#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <deque>
#include <thread>

namespace {

struct PoolSlot {
    FitCtx* c = nullptr;
    int64_t tag = 0;
    long long nsteps = 0;
    long long sched = 0;  // steps enqueued so far
    PoolInst<float> row{};
    cudaEvent_t ready = nullptr;  // end of the caller's work on the context before submit
    bool joined = false;          // the pool stream has waited on `ready`
    double t_submit = 0.0, t_start = -1.0;
    long long pre_steps = 0;  // steps taken at submission (the odd first step of a fused context)
    bool cancel = false;      // fit_pool_cancel: no further chunks; reported once none is in flight
    int inflight = 0;         // chunks in flight that step this context
};

struct InFlight {
    int buf = 0;
    std::vector<PoolSlot*> members;    // every context the chunk steps
    std::vector<PoolSlot*> finishing;  // those whose last steps it takes
    double t_launch = 0.0;
};

}  // namespace

struct FitPool {
    int device = 0;
    int nsm = 1;
    int chunk = 64;
    int ctas_per_sm = 0;
    int minb[3]{3, 3, 4};          // kernel variant (CTAs per SM of its register budget) per class
    int grid_h[3]{}, grid_e[3]{};  // persistent CTAs of the pass kernels per vector class
    int fminb[3]{3, 3, 4};         // fused kernel variant (CTAs per SM) per vector width 4, 2, 1
    int grid_f[3]{};               // persistent CTAs of the fused kernels (4-, 2-, 1-wide vectors)
    int gen = 0;                   // bumped by fit_pool_tune: captured graphs of older variants are stale
    cudaStream_t ps = nullptr;     // every chunk runs here
    cudaEvent_t ev[2]{};
    PoolTable<float>* d_tab[2]{};
    PoolTable<float>* h_tab[2]{};
    cudaGraphExec_t graph[2][1 << kPoolClasses]{};  // [table][mask of the classes present]
    int graph_gen[2][1 << kPoolClasses]{};
    long long budget = 0, reserved = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<PoolSlot*> incoming;
    std::vector<PoolSlot*> active;
    std::deque<FitPoolDone> done;
    std::thread th;
    bool stop = false;
    int status = FIT_OK;
    std::string err;
    long long chunks = 0, cell_updates = 0, fused_cell_updates = 0;
    int max_active = 0;
    double busy_ms = 0.0;
    std::chrono::steady_clock::time_point t0;

    double now() const {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

int pool_fail(FitPool* p, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (p) {
        std::lock_guard<std::mutex> lk(p->mu);
        p->err = buf;
    } else {
        std::lock_guard<std::mutex> lk(g_err_mu);
        g_create_error = buf;
    }
    return code;
}

void finish_slot(FitPool* p, PoolSlot* s, int status, double t) {
    // caller holds p->mu
    FitPoolDone d{};
    d.tag = s->tag;
    d.steps = status == FIT_OK ? s->nsteps + s->pre_steps : 0;
    d.status = status;
    d.t_submit_ms = s->t_submit;
    d.t_start_ms = s->t_start;
    d.t_done_ms = t;
    p->done.push_back(d);
    if (s->ready) cudaEventDestroy(s->ready);
    s->c->in_pool = false;
    delete s;
}

// stops the pool on a CUDA error: every member and queued context is reported failed
void pool_abort(FitPool* p, cudaError_t e, const char* what) {
    std::lock_guard<std::mutex> lk(p->mu);
    char buf[384];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    p->err = buf;
    p->status = FIT_ERR_CUDA;
    const double t = p->now();
    for (PoolSlot* s : p->active) finish_slot(p, s, FIT_ERR_CUDA, t);
    p->active.clear();
    for (PoolSlot* s : p->incoming) finish_slot(p, s, FIT_ERR_CUDA, t);
    p->incoming.clear();
    p->cv_done.notify_all();
}

// active contexts cancelled by fit_pool_cancel that no chunk in flight steps any more are
// handed back with FIT_ERR_CANCELLED (caller holds p->mu)
void retire_cancelled(FitPool* p, double t) {
    bool any = false;
    for (size_t i = 0; i < p->active.size();) {
        PoolSlot* s = p->active[i];
        if (s->cancel && s->inflight == 0) {
            p->active.erase(p->active.begin() + i);
            finish_slot(p, s, FIT_ERR_CANCELLED, t);
            any = true;
        } else {
            ++i;
        }
    }
    if (any) p->cv_done.notify_all();
}

// planes per work item of the fused members of a chunk: about kSegWaves work items per
// CTA of the persistent fused grid, so the last wave of a step is a small part of it,
// within [kSegZlenMin, kSegZlenMax] (a range start recomputes one plane of H)
constexpr int kSegWaves = 4;
constexpr int kSegZlenMin = 8;
constexpr int kSegZlenMax = 64;

int seg_zlen(const FitPool* p, const std::vector<PoolSlot*>& members) {
    long long units = 0;  // segment-planes of the fused members
    for (const PoolSlot* s : members)
        if (s->row.fused) units += s->row.nseg * s->c->g.nz;
    const long long grid = std::max({p->grid_f[0], p->grid_f[1], p->grid_f[2], 1});
    const long long z = units / (kSegWaves * grid);
    return (int)std::min<long long>(kSegZlenMax, std::max<long long>(kSegZlenMin, z));
}

// fills pinned table `b` with the members that still have steps to enqueue, ordered by
// vector class; returns the mask of the classes present
int stage_table(FitPool* p, int b, const std::vector<PoolSlot*>& members) {
    PoolTable<float>* t = p->h_tab[b];
    long long tile = 0;
    int n = 0, mask = 0;
    const int zlen = seg_zlen(p, members);
    for (int cls = 0; cls < kPoolClasses; ++cls) {
        t->cls_t0[cls] = tile;
        for (PoolSlot* s : members) {
            const int sc = s->row.fused ? pool_fused_class(s->row.vec) : pool_class(s->row.vec);
            if (sc != cls) continue;
            PoolInst<float>& r = t->inst[n++];
            r = s->row;
            r.n0c = r.n_end - s->nsteps + s->sched;  // the pooled steps are [n_end - nsteps, n_end)
            if (r.fused) {
                r.zlen = zlen;
                r.ntile = r.nseg * ((r.g.nz + zlen - 1) / zlen);
            }
            r.tile0 = tile;
            tile += r.ntile;
            mask |= 1 << cls;
        }
    }
    t->cls_t0[kPoolClasses] = tile;
    t->ninst = n;
    return mask;
}

// the pooled fused step serves coded FP32 contexts with the fused step enabled (second
// field buffers), the elided J, no plane source or ABC update, and Nx <= kSegMaxNx; any
// Nx % vec == 0 vector width (odd Nx: single cells)
bool pool_fused_ok(const FitCtx* c, int mode) {
    return c->fused && c->E2 && c->H2 && mode != 2 && !c->plane.active && !c->abc_axes && c->d_code && c->d_tab &&
           c->g.nx <= kSegMaxNx;
}

// compiled variants: launch bound (CTAs per SM) choices per vector class
constexpr int kPoolMinb[3][2] = {{2, 3}, {3, 4}, {3, 4}};

bool pool_minb_ok(int cls, int minb) { return minb == kPoolMinb[cls][0] || minb == kPoolMinb[cls][1]; }

template <int VEC, int MINB>
cudaError_t pool_occupancy(int* h, int* e) {
    cudaError_t r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(h, k_hpass_pool<float, VEC, MINB>, kPoolTpb, 0);
    if (r == cudaSuccess) r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(e, k_epass_pool<float, VEC, MINB>, kPoolTpb, 0);
    return r;
}

// persistent grids of class cls with variant minb (capped by ctas_per_sm when set)
cudaError_t pool_grids(int nsm, int cls, int minb, int ctas_per_sm, int* gh, int* ge) {
    int oh = 0, oe = 0;
    cudaError_t e;
    if (cls == 0)
        e = minb == 2 ? pool_occupancy<4, 2>(&oh, &oe) : pool_occupancy<4, 3>(&oh, &oe);
    else if (cls == 1)
        e = minb == 3 ? pool_occupancy<2, 3>(&oh, &oe) : pool_occupancy<2, 4>(&oh, &oe);
    else
        e = minb == 3 ? pool_occupancy<1, 3>(&oh, &oe) : pool_occupancy<1, 4>(&oh, &oe);
    oh = std::max(oh, 1);
    oe = std::max(oe, 1);
    *gh = nsm * (ctas_per_sm ? std::min(ctas_per_sm, oh) : oh);
    *ge = nsm * (ctas_per_sm ? std::min(ctas_per_sm, oe) : oe);
    return e;
}

struct PoolTune {
    int minb[3], grid_h[3], grid_e[3], fminb[3], grid_f[3], gen;
};

// the pooled fused kernel of vector width vec, compiled with the register budgets of m
// CTAs per SM: vec 4: 2 or 3, vec 2 and 1: 3 or 4
constexpr int kSegMinb[3][2] = {{2, 3}, {3, 4}, {3, 4}};
bool pool_fminb_ok(int vec, int m) {
    const int f = vec == 4 ? 0 : (vec == 2 ? 1 : 2);
    return m == kSegMinb[f][0] || m == kSegMinb[f][1];
}
const void* pool_seg_func(int vec, int m) {
    if (vec == 4)
        return m == 2 ? (const void*)k_step_seg_pool<float, 4, 2> : (const void*)k_step_seg_pool<float, 4, 3>;
    if (vec == 2)
        return m == 3 ? (const void*)k_step_seg_pool<float, 2, 3> : (const void*)k_step_seg_pool<float, 2, 4>;
    return m == 3 ? (const void*)k_step_seg_pool<float, 1, 3> : (const void*)k_step_seg_pool<float, 1, 4>;
}

// persistent CTAs of the fused kernel of vector width vec with variant m
cudaError_t pool_grid_f(int nsm, int vec, int m, int ctas_per_sm, int* grid) {
    int of = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&of, pool_seg_func(vec, m), kSegTpb, 0);
    of = std::max(of, 1);
    *grid = nsm * (ctas_per_sm ? std::min(ctas_per_sm, of) : of);
    return e;
}

// kernel entry of class cls's pass with variant m
const void* pool_pass_func(int cls, int m, bool e_pass) {
    if (cls == 0)
        return e_pass ? (m == 2 ? (const void*)k_epass_pool<float, 4, 2> : (const void*)k_epass_pool<float, 4, 3>)
                      : (m == 2 ? (const void*)k_hpass_pool<float, 4, 2> : (const void*)k_hpass_pool<float, 4, 3>);
    if (cls == 1)
        return e_pass ? (m == 3 ? (const void*)k_epass_pool<float, 2, 3> : (const void*)k_epass_pool<float, 2, 4>)
                      : (m == 3 ? (const void*)k_hpass_pool<float, 2, 3> : (const void*)k_hpass_pool<float, 2, 4>);
    return e_pass ? (m == 3 ? (const void*)k_epass_pool<float, 1, 3> : (const void*)k_epass_pool<float, 1, 4>)
                  : (m == 3 ? (const void*)k_hpass_pool<float, 1, 3> : (const void*)k_hpass_pool<float, 1, 4>);
}

// a kernel node that depends on the non-null nodes of deps (graphs are built node by
// node, not captured, so building one never interferes with device-wide synchronisation
// by other threads)
cudaError_t add_node_after(cudaGraph_t g, cudaGraphNode_t* out, const void* func, int grid, dim3 block, void** args,
                           const cudaGraphNode_t* deps, int ndeps) {
    cudaGraphNode_t d[8];
    int n = 0;
    for (int i = 0; i < ndeps && n < 8; ++i)
        if (deps[i]) d[n++] = deps[i];
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void*>(func);
    kp.gridDim = dim3((unsigned)grid);
    kp.blockDim = block;
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    kp.extra = nullptr;
    return cudaGraphAddKernelNode(out, g, n ? d : nullptr, n, &kp);
}

// the graph of table b with the classes in mask: chunk_steps x [taps + counters, the H
// pass of each two-pass class present, their E passes, the fused step of each fused
// class present (direction alternating with the step)].  The classes hold different
// solves, so their kernels are independent branches and overlap (one class's last wave
// with another's work): step s's H pass of a class waits only for that class's E pass
// of step s-1; an E pass or fused step waits for its H pass (fused: its previous step)
// and for the step's prologue, which reads the E it overwrites; the prologue waits for
// the whole previous step (it reads the new E and adds to the tap sums in order).
cudaError_t pool_graph(FitPool* p, const PoolTune& t, int b, int mask, cudaGraphExec_t* out) {
    if (p->graph[b][mask] && p->graph_gen[b][mask] == t.gen) {
        *out = p->graph[b][mask];
        return cudaSuccess;
    }
    if (p->graph[b][mask]) {
        cudaGraphExecDestroy(p->graph[b][mask]);
        p->graph[b][mask] = nullptr;
    }
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaGraphCreate(&gr, 0);
    PoolTable<float>* tab = p->d_tab[b];
    cudaGraphNode_t pro = nullptr, ep[3] = {}, fs[3] = {};  // the previous step's nodes
    for (int s = 0; s < p->chunk && e == cudaSuccess; ++s) {
        int dir = s & 1;
        void* pro_args[3] = {&tab, &dir, &s};
        const cudaGraphNode_t pro_deps[7] = {pro, ep[0], ep[1], ep[2], fs[0], fs[1], fs[2]};
        cudaGraphNode_t pro_s = nullptr;
        e = add_node_after(gr, &pro_s, (const void*)k_prologue_pool<float>, kPoolMaxInst * kPoolProSlices, dim3(256),
                           pro_args, pro_deps, 7);
        void* pass_args[2] = {&tab, &s};
        for (int cls = 0; cls < 3 && e == cudaSuccess; ++cls) {
            if (!(mask & (1 << cls))) continue;
            cudaGraphNode_t h = nullptr;
            e = add_node_after(gr, &h, pool_pass_func(cls, t.minb[cls], false), t.grid_h[cls], dim3(kPoolTpb),
                               pass_args, &ep[cls], 1);
            const cudaGraphNode_t e_deps[2] = {h, pro_s};
            if (e == cudaSuccess)
                e = add_node_after(gr, &ep[cls], pool_pass_func(cls, t.minb[cls], true), t.grid_e[cls],
                                   dim3(kPoolTpb), pass_args, e_deps, 2);
        }
        void* fused_args[3] = {&tab, &dir, &s};
        for (int f = 0; f < 3 && e == cudaSuccess; ++f) {
            if (!(mask & (1 << (3 + f)))) continue;
            const cudaGraphNode_t f_deps[2] = {fs[f], pro_s};
            e = add_node_after(gr, &fs[f], pool_seg_func(4 >> f, t.fminb[f]), t.grid_f[f], dim3(kSegTpb), fused_args,
                               f_deps, 2);
        }
        pro = pro_s;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->graph[b][mask], gr, 0);
    if (gr) cudaGraphDestroy(gr);
    if (e == cudaSuccess) {
        p->graph_gen[b][mask] = t.gen;
        *out = p->graph[b][mask];
    }
    return e;
}

// kernel launches of one step of a chunk with the classes in mask
int pool_launches_per_step(int mask) {
    int n = 1;
    for (int c = 0; c < 3; ++c) n += 2 * ((mask >> c) & 1);
    for (int c = 3; c < kPoolClasses; ++c) n += (mask >> c) & 1;
    return n;
}


void pool_main(FitPool* p) {
    if (cudaSetDevice(p->device) != cudaSuccess) {
        pool_abort(p, cudaErrorInvalidDevice, "cudaSetDevice");
        return;
    }
    std::deque<InFlight> fl;
    long long k = 0;
    double busy_since = -1.0;
    for (;;) {
        std::vector<PoolSlot*> members;
        bool launch = false;
        PoolTune tune{};
        {
            std::unique_lock<std::mutex> lk(p->mu);
            if (p->stop && fl.empty()) break;
            if (!p->stop && fl.empty() && p->active.empty() && p->incoming.empty()) {
                p->cv_work.wait(lk, [p] { return p->stop || !p->incoming.empty(); });
                continue;
            }
            if (!p->stop) {
                retire_cancelled(p, p->now());
                while (!p->incoming.empty() && (int)p->active.size() < kPoolMaxInst) {
                    p->active.push_back(p->incoming.front());
                    p->incoming.pop_front();
                }
                for (PoolSlot* s : p->active)
                    if (s->sched < s->nsteps && !s->cancel) members.push_back(s);
                launch = !members.empty() && fl.size() < 2;
                for (int c = 0; c < 3; ++c) {
                    tune.minb[c] = p->minb[c];
                    tune.grid_h[c] = p->grid_h[c];
                    tune.grid_e[c] = p->grid_e[c];
                }
                for (int f = 0; f < 3; ++f) {
                    tune.fminb[f] = p->fminb[f];
                    tune.grid_f[f] = p->grid_f[f];
                }
                tune.gen = p->gen;
            }
        }
        if (launch) {
            const int b = (int)(k & 1);
            const int mask = stage_table(p, b, members);
            const int n = (int)members.size();
            cudaGraphExec_t gx = nullptr;
            cudaError_t e = pool_graph(p, tune, b, mask, &gx);
            for (PoolSlot* s : members)
                if (!s->joined && e == cudaSuccess) {
                    e = cudaStreamWaitEvent(p->ps, s->ready, 0);
                    s->joined = true;
                }
            const size_t bytes = offsetof(PoolTable<float>, inst) + (size_t)n * sizeof(PoolInst<float>);
            if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_tab[b], p->h_tab[b], bytes, cudaMemcpyHostToDevice, p->ps);
            if (e == cudaSuccess) e = cudaGraphLaunch(gx, p->ps);
            if (e == cudaSuccess) e = cudaEventRecord(p->ev[b], p->ps);
            if (e != cudaSuccess) {
                pool_abort(p, e, "pool chunk launch");
                break;
            }
            g_launches += (long long)pool_launches_per_step(mask) * p->chunk;
            InFlight f;
            f.buf = b;
            f.t_launch = p->now();
            if (busy_since < 0) busy_since = f.t_launch;
            long long cells = 0, fcells = 0;
            {
                std::lock_guard<std::mutex> lk(p->mu);  // inflight is read by retire_cancelled
                for (PoolSlot* s : members) {
                    const long long take = std::min<long long>(p->chunk, s->nsteps - s->sched);
                    if (s->t_start < 0) s->t_start = f.t_launch;
                    s->sched += take;
                    s->inflight++;
                    cells += take * s->c->g.N;
                    if (s->row.fused) fcells += take * s->c->g.N;
                    if (s->sched >= s->nsteps) f.finishing.push_back(s);
                }
            }
            f.members = members;
            {
                std::lock_guard<std::mutex> lk(p->mu);
                p->chunks++;
                p->cell_updates += cells;
                p->fused_cell_updates += fcells;
                p->max_active = std::max(p->max_active, n);
            }
            fl.push_back(std::move(f));
            ++k;
            continue;
        }
        // wait for the oldest chunk in flight
        InFlight f = std::move(fl.front());
        fl.pop_front();
        cudaError_t e = cudaEventSynchronize(p->ev[f.buf]);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) {
            pool_abort(p, e, "pool chunk");
            break;
        }
        const double t = p->now();
        std::lock_guard<std::mutex> lk(p->mu);
        if (fl.empty()) {
            p->busy_ms += t - busy_since;
            busy_since = -1.0;
        }
        for (PoolSlot* s : f.members) s->inflight--;
        for (PoolSlot* s : f.finishing) {
            p->active.erase(std::remove(p->active.begin(), p->active.end(), s), p->active.end());
            finish_slot(p, s, FIT_OK, t);
        }
        if (!f.finishing.empty()) p->cv_done.notify_all();
        retire_cancelled(p, t);
    }
    // stopping: what is still in the pool is handed back unfinished
    std::lock_guard<std::mutex> lk(p->mu);
    const double t = p->now();
    for (PoolSlot* s : p->active) finish_slot(p, s, FIT_ERR_STATE, t);
    p->active.clear();
    for (PoolSlot* s : p->incoming) finish_slot(p, s, FIT_ERR_STATE, t);
    p->incoming.clear();
    p->cv_done.notify_all();
}

void pool_free(FitPool* p) {
    cudaSetDevice(p->device);
    if (p->ps) cudaStreamSynchronize(p->ps);
    for (int b = 0; b < 2; ++b) {
        for (int m = 0; m < (1 << kPoolClasses); ++m)
            if (p->graph[b][m]) cudaGraphExecDestroy(p->graph[b][m]);
        if (p->ev[b]) cudaEventDestroy(p->ev[b]);
        if (p->d_tab[b]) cudaFree(p->d_tab[b]);
        if (p->h_tab[b]) cudaFreeHost(p->h_tab[b]);
    }
    if (p->ps) cudaStreamDestroy(p->ps);
    delete p;
}

}  // namespace

extern "C" {

int fit_pool_create(int32_t device, int64_t budget_bytes, int32_t chunk_steps, int32_t ctas_per_sm, FitPool** out) {
    if (!out) return pool_fail(nullptr, FIT_ERR_ARG, "null argument");
    *out = nullptr;
    if (budget_bytes <= 0) return pool_fail(nullptr, FIT_ERR_ARG, "budget_bytes must be > 0");
    if (chunk_steps < 1 || chunk_steps > 1024) return pool_fail(nullptr, FIT_ERR_ARG, "chunk_steps must be in [1, 1024]");
    if (ctas_per_sm < 0 || ctas_per_sm > 32) return pool_fail(nullptr, FIT_ERR_ARG, "ctas_per_sm must be in [0, 32]");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return pool_fail(nullptr, FIT_ERR_DEVICE, "no CUDA device available");
    if (device < 0 || device >= ndev) return pool_fail(nullptr, FIT_ERR_ARG, "invalid device %d", device);
    FitPool* p = new FitPool();
    p->device = device;
    p->budget = budget_bytes;
    p->chunk = chunk_steps;
    p->t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, device);
    p->ctas_per_sm = ctas_per_sm;
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = pool_grids(p->nsm, c, p->minb[c], ctas_per_sm, &p->grid_h[c], &p->grid_e[c]);
    for (int f = 0; f < 3 && e == cudaSuccess; ++f) e = pool_grid_f(p->nsm, 4 >> f, p->fminb[f], ctas_per_sm, &p->grid_f[f]);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->ps, cudaStreamNonBlocking);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        e = cudaEventCreateWithFlags(&p->ev[b], cudaEventDisableTiming | cudaEventBlockingSync);
        if (e == cudaSuccess) e = cudaMalloc(&p->d_tab[b], sizeof(PoolTable<float>));
        if (e == cudaSuccess) e = cudaMemset(p->d_tab[b], 0, sizeof(PoolTable<float>));
        if (e == cudaSuccess) e = cudaMallocHost(&p->h_tab[b], sizeof(PoolTable<float>));
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->ps);
    if (e != cudaSuccess) {
        int rc = pool_fail(nullptr, FIT_ERR_CUDA, "pool setup failed: %s", cudaGetErrorString(e));
        pool_free(p);
        return rc;
    }
    p->th = std::thread(pool_main, p);
    *out = p;
    return FIT_OK;
}

int fit_pool_destroy(FitPool* p) {
    if (!p) return FIT_OK;
    {
        std::lock_guard<std::mutex> lk(p->mu);
        p->stop = true;
    }
    p->cv_work.notify_all();
    if (p->th.joinable()) p->th.join();
    pool_free(p);
    return FIT_OK;
}

int fit_pool_last_error(const FitPool* p, char* buf, int64_t len) {
    if (!buf || len <= 0) return FIT_ERR_ARG;
    std::string m;
    if (p) {
        std::lock_guard<std::mutex> lk(const_cast<FitPool*>(p)->mu);
        m = p->err;
    } else {
        std::lock_guard<std::mutex> lk(g_err_mu);
        m = g_create_error;
    }
    snprintf(buf, (size_t)len, "%s", m.c_str());
    return FIT_OK;
}

int fit_pool_reserve(FitPool* p, int64_t bytes) {
    if (!p || bytes < 0) return FIT_ERR_ARG;
    std::lock_guard<std::mutex> lk(p->mu);
    if (bytes > p->budget) {
        p->err = "reservation larger than the pool budget";
        return FIT_ERR_ARG;
    }
    if (p->reserved + bytes > p->budget) return FIT_ERR_BUDGET;
    p->reserved += bytes;
    return FIT_OK;
}

int fit_pool_release(FitPool* p, int64_t bytes) {
    if (!p || bytes < 0) return FIT_ERR_ARG;
    std::lock_guard<std::mutex> lk(p->mu);
    if (bytes > p->reserved) {
        p->err = "release of more bytes than reserved";
        return FIT_ERR_ARG;
    }
    p->reserved -= bytes;
    return FIT_OK;
}

int fit_pool_submit(FitPool* p, FitCtx* c, int64_t n0, int64_t nsteps, int64_t tag) {
    if (!p || !c) return FIT_ERR_ARG;
    int rc = check_ready(c);
    if (rc) return rc;
    if (c->in_pool) return fail(c, FIT_ERR_STATE, "the context is already in a pool");
    if (c->device != p->device) return fail(c, FIT_ERR_ARG, "context and pool are on different devices");
    if (c->dtype != FIT_F32) return fail(c, FIT_ERR_ARG, "the pool steps FP32 contexts");
    if (c->plane.active || c->abc_axes) return fail(c, FIT_ERR_ARG, "plane sources and ABC updates are not pooled");
    if (n0 < 0 || nsteps <= 0) return fail(c, FIT_ERR_ARG, "bad step range");
    if (c->beam.active && (!c->beam.dtieps || c->vt_len < n0 + nsteps))
        return fail(c, FIT_ERR_STATE, "beam v*t table shorter than the run (%lld < %lld)", c->vt_len,
                    (long long)(n0 + nsteps));
    {
        std::lock_guard<std::mutex> lk(p->mu);
        if (p->status != FIT_OK) return fail(c, p->status, "the pool stopped: %s", p->err.c_str());
        if (p->stop) return fail(c, FIT_ERR_STATE, "the pool is stopping");
    }
    rc = enter(c);  // orders the caller's stream before the context stream
    if (rc) return rc;
    static thread_local long long host_n0;
    host_n0 = n0;
    CK(cudaMemcpyAsync(c->d_step, &host_n0, sizeof(long long), cudaMemcpyHostToDevice, c->own));
    // a coded context with the fused step enabled is stepped by the pooled fused kernel
    // (when the chunk length is even); it takes its steps in pairs (ending in E, H), so an
    // odd count takes its first step here with the two-pass kernels
    const int mode = c->use_cond ? 1 : 0;
    const bool fused = pool_fused_ok(c, mode) && p->chunk % 2 == 0;
    long long pooled = nsteps;
    if (fused && (nsteps % 2)) {
        launch_step(c, 0, mode, true);
        pooled -= 1;
    }
    PoolSlot* s = new PoolSlot();
    cudaError_t e = cudaEventCreateWithFlags(&s->ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(s->ready, c->own);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->own);  // host_n0 is read before it changes
    if (e != cudaSuccess) {
        if (s->ready) cudaEventDestroy(s->ready);
        delete s;
        return fail(c, FIT_ERR_CUDA, "pool submit: %s", cudaGetErrorString(e));
    }
    s->c = c;
    s->tag = tag;
    s->nsteps = pooled;
    s->pre_steps = nsteps - pooled;
    PoolInst<float>& r = s->row;
    r.g = c->g;
    r.mt = metric<float>(c);
    r.E = static_cast<float*>(c->E);
    r.H = static_cast<float*>(c->H);
    r.ch = static_cast<const float*>(c->ch);
    r.ce = static_cast<const float*>(c->ce);
    r.cl = static_cast<const float*>(c->cl);
    r.J = static_cast<float*>(c->J);
    // every class reads the context's coefficient codes when it has them (the fused
    // class only takes coded contexts)
    r.code = c->d_code;
    r.tab = static_cast<const float*>(c->d_tab);
    r.beam = c->beam;
    r.tap = c->tap;
    r.d_step = c->d_step;
    r.vt_table = c->d_vt_table;
    r.vt_len = c->vt_len;
    r.n_end = n0 + nsteps;
    r.vec = pick_vec(c);
    // odd Nx with N even and coded coefficients: the 1-wide class steps cell pairs
    r.pair = (r.vec == 1 && c->g.N % 2 == 0 && c->d_code && c->d_tab) ? 1 : 0;
    r.nvec = r.pair ? c->g.N / 2 : c->g.N / r.vec;
    r.mode = c->use_cond ? 1 : 0;
    r.use_cond = c->use_cond;
    r.ntile = (r.nvec + kPoolTpb - 1) / kPoolTpb;
    if (fused) {
        r.fused = 1;
        r.E2 = static_cast<float*>(c->E2);
        r.H2 = static_cast<float*>(c->H2);
        r.nseg = (c->g.sz + (kSegWin - c->g.nx) - 1) / (kSegWin - c->g.nx);
        r.zlen = kSegZlenMax;  // set per chunk by stage_table
        r.ntile = r.nseg * ((c->g.nz + r.zlen - 1) / r.zlen);
    }
    c->in_pool = true;
    {
        std::lock_guard<std::mutex> lk(p->mu);
        s->t_submit = p->now();
        p->incoming.push_back(s);
    }
    p->cv_work.notify_all();
    return FIT_OK;
}

int fit_pool_cancel(FitPool* p, int64_t tag) {
    if (!p) return FIT_ERR_ARG;
    std::lock_guard<std::mutex> lk(p->mu);
    for (auto it = p->incoming.begin(); it != p->incoming.end(); ++it) {
        if ((*it)->tag == tag) {
            PoolSlot* s = *it;
            p->incoming.erase(it);
            finish_slot(p, s, FIT_ERR_CANCELLED, p->now());
            p->cv_done.notify_all();
            return FIT_OK;
        }
    }
    for (PoolSlot* s : p->active) {
        if (s->tag == tag) {  // a repeated cancel is a no-op
            s->cancel = true;
            p->cv_work.notify_all();
            return FIT_OK;
        }
    }
    p->err = "fit_pool_cancel: no queued or running solve with tag " + std::to_string((long long)tag);
    return FIT_ERR_ARG;
}

int fit_pool_poll(FitPool* p, FitPoolDone* out, int32_t max, int32_t wait_ms) {
    if (!p || (!out && max > 0) || max < 0) return FIT_ERR_ARG;
    std::unique_lock<std::mutex> lk(p->mu);
    if (p->done.empty() && wait_ms > 0 && (!p->active.empty() || !p->incoming.empty()))
        p->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [p] { return !p->done.empty(); });
    int n = 0;
    while (n < max && !p->done.empty()) {
        out[n++] = p->done.front();
        p->done.pop_front();
    }
    return n;
}

int fit_pool_tune(FitPool* p, int32_t vec, int32_t ctas_per_sm) {
    if (!p || (vec != 4 && vec != 2 && vec != 1)) return FIT_ERR_ARG;
    const int cls = pool_class(vec);
    if (!pool_minb_ok(cls, ctas_per_sm)) {
        std::lock_guard<std::mutex> lk(p->mu);
        p->err = "no compiled pool kernel variant for that vector width and CTAs per SM";
        return FIT_ERR_ARG;
    }
    int gh = 0, ge = 0;
    cudaError_t e = cudaSetDevice(p->device);
    if (e == cudaSuccess) e = pool_grids(p->nsm, cls, ctas_per_sm, p->ctas_per_sm, &gh, &ge);
    if (e != cudaSuccess) return pool_fail(p, FIT_ERR_CUDA, "fit_pool_tune: %s", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(p->mu);
    p->minb[cls] = ctas_per_sm;
    p->grid_h[cls] = gh;
    p->grid_e[cls] = ge;
    p->gen++;
    return FIT_OK;
}

int fit_pool_tune_fused(FitPool* p, int32_t vec, int32_t ctas_per_sm) {
    if (!p || (vec != 4 && vec != 2 && vec != 1)) return FIT_ERR_ARG;
    if (!pool_fminb_ok(vec, ctas_per_sm)) {
        std::lock_guard<std::mutex> lk(p->mu);
        p->err = "no compiled fused pool kernel variant for that vector width and CTAs per SM";
        return FIT_ERR_ARG;
    }
    const int f = vec == 4 ? 0 : (vec == 2 ? 1 : 2);
    int gf = 0;
    cudaError_t e = cudaSetDevice(p->device);
    if (e == cudaSuccess) e = pool_grid_f(p->nsm, vec, ctas_per_sm, p->ctas_per_sm, &gf);
    if (e != cudaSuccess) return pool_fail(p, FIT_ERR_CUDA, "fit_pool_tune_fused: %s", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(p->mu);
    p->fminb[f] = ctas_per_sm;
    p->grid_f[f] = gf;
    p->gen++;
    return FIT_OK;
}

int fit_pool_stats(FitPool* p, FitPoolStats* out) {
    if (!p || !out) return FIT_ERR_ARG;
    std::lock_guard<std::mutex> lk(p->mu);
    FitPoolStats s{};
    s.chunks = p->chunks;
    s.cell_updates = p->cell_updates;
    s.budget_bytes = p->budget;
    s.reserved_bytes = p->reserved;
    s.active = (int32_t)p->active.size();
    s.queued = (int32_t)p->incoming.size();
    s.max_active = p->max_active;
    for (int c = 0; c < 3; ++c) {
        s.variant[c] = p->minb[c];
        s.grid[c] = p->grid_e[c];
    }
    s.chunk_steps = p->chunk;
    s.busy_ms = p->busy_ms;
    s.fused_cell_updates = p->fused_cell_updates;
    for (int f = 0; f < 3; ++f) {
        s.fused_variant[f] = p->fminb[f];
        s.fused_grid[f] = p->grid_f[f];
    }
    *out = s;
    return FIT_OK;
}

}  // extern "C"
