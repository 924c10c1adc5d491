/*
 * wakis_fit.h -- C ABI of the GB300 (sm_103a) Finite Integration Technique leapfrog path.
 *
 * One context (FitCtx) holds one rectilinear grid: the caller-owned field storage
 * E, H, J (device pointers, 3*N elements each, component blocks [x | y | z], each block
 * in Fortran order n = i + Nx*j + Nx*Ny*k), the library-owned per-edge / per-face
 * coefficient arrays, the optional fused sources (beam line current, hard plane
 * source), the optional wake-potential line taps and the step machinery.
 *
 * Every entry point returns 0 (FIT_OK) or a negative FIT_ERR_* code; the message of
 * the last failure is available through fit_last_error().  Device faults are never
 * turned into traps: kernels write error codes that the host reads.
 *
 * Pointers documented as "device" must be CUDA device pointers on the context's
 * device; "host" pointers are plain host memory read during the call.
 * Citations name the reference interface (Wakis 0.7.0) each entry point replaces.
 */
#ifndef WAKIS_FIT_H
#define WAKIS_FIT_H

#include <stdint.h>

#if defined(__GNUC__)
#define FIT_API __attribute__((visibility("default")))
#else
#define FIT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define FIT_OK 0
#define FIT_ERR_ARG (-1)
#define FIT_ERR_CUDA (-2)
#define FIT_ERR_STATE (-3)
#define FIT_ERR_TIMEOUT (-4)
#define FIT_ERR_NOMEM (-5)
#define FIT_ERR_DEVICE (-6)
#define FIT_ERR_BUDGET (-7) /* a pool reservation would exceed the pool's memory budget */
#define FIT_ERR_CANCELLED (-8) /* a pooled solve was cancelled (fit_pool_cancel) */

#define FIT_F32 0
#define FIT_F64 1

/* boundary codes per face (wakis/boundaries.py:14-188) */
#define FIT_BC_PERIODIC 0
#define FIT_BC_PEC 1 /* 'pec' or 'electric' */
#define FIT_BC_PML 2
#define FIT_BC_PMC 3 /* 'pmc' or 'magnetic' */
#define FIT_BC_ABC 4

/* E-pass variants: how the conduction current J enters the E update
 * (wakis/solverFIT3D.py:514-525). */
#define FIT_J_ELIDED 0   /* J == sigma*E of the previous step (or 0): folded into a loss factor */
#define FIT_J_EXPLICIT 1 /* J read from storage; J = sigma*E written back when conductive */
#define FIT_STEP_NO_BEAM 2 /* or-ed into j_mode: the beam line current is off for this step */

typedef struct FitCtx FitCtx;

typedef struct FitGridDesc {
    int64_t nx, ny, nz;
    int32_t dtype;            /* FIT_F32 or FIT_F64: storage and stencil arithmetic */
    int32_t use_conductivity; /* SolverFIT3D.use_conductivity */
    int32_t bc_lo[3];         /* FIT_BC_* for the x, y, z low faces */
    int32_t bc_hi[3];         /* FIT_BC_* for the x, y, z high faces */
    int32_t device;           /* CUDA device ordinal */
    int32_t reserved;
    void *E, *H, *J; /* device, 3*N elements of dtype each (caller-owned) */
} FitGridDesc;

/* Context lifetime.  Replaces the operator assembly of SolverFIT3D.__init__
 * (wakis/solverFIT3D.py:203-227, 337-344): no sparse matrix is built.  Grids with
 * N + Nx*Ny >= 2^31 (N = Nx*Ny*Nz) are refused with FIT_ERR_ARG: the kernels address
 * cells by 32-bit offsets within a field component. */
FIT_API int fit_ctx_create(const FitGridDesc *desc, FitCtx **out);
FIT_API int fit_ctx_destroy(FitCtx *ctx);
/* Copies the last error message (NUL terminated, truncated to len); ctx may be NULL
 * for errors raised by fit_ctx_create. */
FIT_API int fit_last_error(const FitCtx *ctx, char *buf, int64_t len);
/* Stream (cudaStream_t) every later launch of this context is issued on; NULL = legacy. */
FIT_API int fit_set_stream(FitCtx *ctx, void *stream);
/* Rebinds E, H, J (device) after the caller reallocated them. */
FIT_API int fit_set_fields(FitCtx *ctx, void *E, void *H, void *J);

/* Grid metrics (wakis/gridFIT3D.py:263-305): host FP64 arrays of primal edge lengths
 * dx[nx], dy[ny], dz[nz] and UNEDITED dual edge lengths tdx[nx], tdy[ny], tdz[nz]
 * (last entry 0).  Periodic / ABC edits of tL and itA (wakis/boundaries.py:36-70,
 * 153-181) are applied by the library from the face codes. */
FIT_API int fit_set_metrics(FitCtx *ctx, const double *dx, const double *dy, const double *dz,
                    const double *tdx, const double *tdy, const double *tdz);

/* Coefficients from FP64 material tensors (device, 3*N each): ieps = 1/eps, imu = 1/mu,
 * sigma.  Builds, on the device in FP64 and stores in the field dtype,
 *   ch = dt*iA*imu*[PMC row mask]          (H pass, the tDs.iDmu.iDa.C operator)
 *   ce = dt*ieps*itA*[PEC row mask]        (E pass, the itDa.iDeps.C^T.tDs operator)
 *   cl = 1 - dt*ieps*sigma                 (loss factor of the elided-J E pass)
 * (wakis/solverFIT3D.py:337-344, 378-436).  The material arrays are read during the call
 * only, except that FIT_J_EXPLICIT steps keep a dtype copy of dt*ieps and sigma. */
FIT_API int fit_set_coeffs(FitCtx *ctx, double dt, const double *ieps, const double *imu,
                   const double *sigma);
/* Allocates the dtype copies of dt*ieps and sigma that FIT_J_EXPLICIT steps read
 * (J set by the caller, wakis/solverFIT3D.py:514-525); the next fit_set_coeffs fills them. */
FIT_API int fit_enable_explicit_j(FitCtx *ctx);

/* Zeroes the ghost tangential components on the last index planes, as the first
 * one_step does (wakis/solverFIT3D.py:505-508, 842-862). */
FIT_API int fit_zero_ghosts(FitCtx *ctx);

/* Gaussian beam line current J_z(ixs, iys, :) of sources.Beam.update
 * (wakis/sources.py:76-110), evaluated inside the E pass:
 *   J_z(k) = q*v*[exp(-((z_k - vt) - s0)^2 / (2 sigmaz^2)) / sqrt(2 pi sigmaz^2)] / dx / dy
 * z (host, nz cell-centre coordinates), ieps_line (host, nz values of ieps_z on the line).
 * active = 0 removes the beam. */
FIT_API int fit_set_beam(FitCtx *ctx, int32_t active, int32_t ixs, int32_t iys, double q, double v,
                 double sigmaz, double s0, double dx_s, double dy_s, const double *z,
                 const double *ieps_line);
/* Per-step beam position v*t.  Either one value for the next host-driven step, or a
 * table (host, n entries) indexed by the step number for fit_run. */
FIT_API int fit_set_beam_vt(FitCtx *ctx, double vt);
FIT_API int fit_set_beam_vt_table(FitCtx *ctx, const double *vt, int64_t n);

/* Hard plane source of sources.PlaneWave / sources.WavePacket (wakis/sources.py:218-248,
 * 373-420): at step n, before the H pass,
 *   H_y(i, j, zs) = (c1[n] * g[i-x0, j-y0]) * gt[n]  and  E_x(i, j, zs) = (c2[n] * g) * gt[n]
 * for x0 <= i < x1, y0 <= j < y1.  prof (host, (x1-x0)*(y1-y0) values, x fastest) may be
 * NULL for g = 1.  c1, c2, gt (host, n entries each).  active = 0 removes it. */
FIT_API int fit_set_plane_source(FitCtx *ctx, int32_t active, int32_t zs, int32_t x0, int32_t x1,
                         int32_t y0, int32_t y1, const double *prof, const double *c1,
                         const double *c2, const double *gt, int64_t n);

/* First-order ABC of emsolve on the CPU reference (wakis/routines.py:183-220,
 * wakis/boundaries.py:307-404): after each step the index-1 plane of E and H is copied
 * to the index-0 plane for every axis bit set in lo_axes (bit 0 = x, 1 = y, 2 = z). */
FIT_API int fit_set_abc(FitCtx *ctx, int32_t lo_axes);

/* Wake-potential line taps (wakis/wakeSolver.py:423-551).  nlines transverse lines at
 * cells (lx[l], ly[l]) (host); a tap table in CSR over steps (host): entries of step n
 * are row_ptr[n] .. row_ptr[n+1]-1, each adding
 *   sum_{c < cnt} E_z(lx, ly, k0 + c + kskip) * dz[k0 + c]
 * to accumulator (line, m) with FP64 Neumaier compensation.  dz (host, nz_tap values).
 * Replaces the per-step Ez.h5 dump (wakis/routines.py:422-445) and the interpreted
 * integral loop. */
FIT_API int fit_set_wake_taps(FitCtx *ctx, int32_t nlines, const int32_t *lx, const int32_t *ly,
                      int32_t kskip, int32_t ns, int64_t nsteps, const int64_t *row_ptr,
                      const int32_t *ent_m, const int32_t *ent_k0, const int32_t *ent_cnt,
                      int32_t nz_tap, const double *dz);
FIT_API int fit_reset_wake(FitCtx *ctx);
/* Raw line integrals (host out, nlines*ns FP64, line-major). */
FIT_API int fit_read_wake(FitCtx *ctx, double *out);

/* One leapfrog step (wakis/solverFIT3D.py:504-525) at step number n with the given
 * J variant (FIT_J_*, optionally | FIT_STEP_NO_BEAM):
 * [plane source, wake taps at E^n] -> H pass -> E pass (+beam) -> [ABC]. */
FIT_API int fit_step(FitCtx *ctx, int64_t n, int32_t j_mode);
/* nsteps steps n0 .. n0+nsteps-1 with the elided-J E pass, the beam vt taken from the
 * vt table and the step number read on the device (CUDA-graph replay of chunks). */
FIT_API int fit_run(FitCtx *ctx, int64_t n0, int64_t nsteps);

/* Brings the J storage up to date (the J of wakis/solverFIT3D.py:524-525 and
 * wakis/sources.py:108-110): flags bit 0 writes J = sigma*E in the field dtype from FP64
 * sigma (device, 3*N; conductive contexts only), bit 1 then writes the beam line current
 * at the vt of fit_set_beam_vt. */
FIT_API int fit_materialize_J(FitCtx *ctx, const double *sigma, int32_t flags);

/* Wake post-processing on the device in FP64 (wakis/wakeSolver.py:480-611):
 * raw (device-resident accumulators of fit_set_wake_taps) combined line by line as
 * WP_3d[l] = (WP_3d[l-1] + raw[l]) / qscale, then the Panofsky-Wenzel transverse
 * wake from exclusive prefix sums along s (ds) and the central differences over
 * dxf = (dxf0 + dxf1), dyf = (dyf0 + dyf1).  Outputs (host): wp3d (nlines*ns),
 * wpx, wpy (ns each; untouched when nlines != 9). */
FIT_API int fit_wake_finalize(FitCtx *ctx, double qscale, double ds, double dxf, double dyf,
                      double *wp3d, double *wpx, double *wpy);

/* Wake potential from a recorded Ez line history, without a context: the post-processing
 * of an Ez file (WakeSolver.calc_long_WP, wakis/wakeSolver.py:311-421, and
 * calc_long_WP_3d + calc_trans_WP, wakis/wakeSolver.py:423-626).  Inputs (host):
 * ezt (nlines*nz*nt FP64, line-major, each line the reference's Ezt (nz, nt)), it (nz*ns,
 * z-major: the time index of tap (m, k) after the reference's negative-index wrap, -1
 * where the reference skips the tap because it >= nt), dz (nz).  Per s index the sums run
 * in the reference's order with plain FP64 adds of rounded products, continue from the
 * previous line's result, and are divided by qscale after each line, so wp3d equals the
 * reference's WP_3d bit for bit.  Then, when the lines form a square of odd side
 * 2n+1 >= 3 (row-major, the reference's n_transverse_cells = n), the transverse wake as in
 * fit_wake_finalize from lines (n+1, n), (n-1, n), (n, n+1), (n, n-1), with dxf, dyf the
 * sums dxf[n-1] + dxf[n], dyf[n-1] + dyf[n] (wakis/wakeSolver.py:553-611).  Outputs
 * (host): wp3d (nlines*ns); wpx, wpy (ns each; untouched for other line counts or NULL).
 * Errors: fit_last_error(NULL, ...). */
FIT_API int fit_wake_history(const double *ezt, int32_t nlines, int64_t nt, int32_t nz, const int32_t *it,
                             int32_t ns, const double *dz, double qscale, double ds, double dxf, double dyf,
                             double *wp3d, double *wpx, double *wpy);

/* FP64 direct DFT at bins b0 .. b0+nb-1 of an n-point zero-padded transform
 *   X_s[b] = sum_{t < len} x_s[t] exp(-2 pi i b t / n)
 * for nsig signals of length len (host, signal-major); out (host) holds nsig*nb
 * (re, im) pairs.  Replaces np.fft.fft(..., n=N)[mask] (wakis/wakeSolver.py:692-699,
 * 755-770).  Uses library-allocated device scratch for partial sums.  At most 65535
 * signals per call (FIT_ERR_ARG beyond). */
FIT_API int fit_dft(const double *x, int32_t nsig, int64_t len, int64_t n, int64_t b0, int32_t nb,
            double *out);

/* Allocation-free variant of fit_dft; it has no counterpart in the reference.  For callers
 * that cannot allocate device memory when they need a spectrum: a process whose device
 * memory is all owned by its own pool (field storage of many concurrent solves), or one
 * that must not take the device-wide synchronisation of cudaMalloc / cudaFree while
 * kernels run on other streams.  x (device, nsig*len FP64, signal-major) and out (device,
 * nsig*nb (re, im) FP64 pairs) belong to the caller; the work is queued on `stream`
 * (cudaStream_t, NULL = legacy default stream) and the call returns without waiting.
 * Partial sums live in one fixed file-scope device array of 2^18 double2 (4 MiB) that every
 * GPU loading this library holds until the process exits: nsig*nb must not exceed 2^18
 * (FIT_ERR_ARG otherwise), and nsig must not exceed 65535.  x and out must be device (or
 * managed) memory of the current device: other pointers are refused with FIT_ERR_ARG
 * before anything is launched.  The array keeps the last call's contents; every entry a call
 * reads is written earlier in the same call, so nothing is cleared.  All calls on a device
 * share the array: calls that overlap on the GPU race.  The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress) with that device current; make
 * that first call before any stream capture.  Errors: fit_last_error(NULL, ...). */
FIT_API int fit_dft_noalloc(const double *x, int32_t nsig, int64_t len, int64_t n, int64_t b0,
                            int32_t nb, double *out, void *stream);

/* Reads the context's device error word (synchronizes the context stream): FIT_OK, or
 * FIT_ERR_TIMEOUT when a kernel gave up a bounded wait on its bulk copies (the kernel
 * then returned without completing its pass).  The word is cleared by the read. */
FIT_API int fit_check_error(FitCtx *ctx);

/* Chooses the step kernels.  0 (the default): the direct H and E pass kernels.
 * 1: the persistent bulk-copy (staged) pass kernels when Nx*sizeof(dtype) is a multiple
 * of 16 bytes.  2: fit_run takes its steps with the fused single-pass kernel (each value
 * read and written once per step) between the caller's E, H and a second pair of field
 * buffers the library allocates (3*N elements each); pairs of steps end in the caller's
 * buffers, and a single step, plane sources, low-face ABC updates, explicit J and grids
 * with Nx not a multiple of 2 use the pass kernels. */
FIT_API int fit_set_kernel_variant(FitCtx *ctx, int32_t variant);
/* Coded coefficients for the fused step; no counterpart in the reference.  enable != 0:
 * the context finds the distinct per-cell triples (ch, ce, cl) of its coefficient arrays
 * on the device and, when there are at most 65535 of them, stores one 16-bit code per
 * cell and a table of the exact triples; the fused step and the two-pass passes (not the
 * FIT_J_EXPLICIT E pass) then read 2 bytes of coefficients per cell instead of 3 to 9
 * words, with bit-identical results.  Contexts submitted to a pool keep their codes for
 * the pool's two-pass classes.  Every cell's
 * code is checked against its triple before the codes are used.  *ncodes (may be NULL)
 * receives the number of distinct triples, or 0 when the context stays dense (too many
 * triples).  fit_set_coeffs drops the codes; enable == 0 drops them too.  Needs
 * N*2 bytes plus a table of 12 words per code (during the build about 14 MB more). */
FIT_API int fit_set_coeff_codes(FitCtx *ctx, int32_t enable, int32_t *ncodes);

/* Tile shape of the fused step: vec cells per thread along x (2, or 4 for FP32; Nx must
 * be a multiple), rows (4 or 8) rows of 32 threads per CTA, zseg z ranges per tile
 * column (1..Nz), ctas the CTAs per SM its register budget is sized for (8 rows: 2;
 * 4 rows: 3 or 4; 0 = the first).  fit_set_kernel_variant(ctx, 2) sets a default; the
 * solver's autotuner times the candidates on the grid itself with fit_time_fused. */
FIT_API int fit_set_fused_shape(FitCtx *ctx, int32_t vec, int32_t rows, int32_t zseg, int32_t ctas);
/* How the fused step's old fields reach the threads (same results bit for bit):
 * staging 0 = per-thread global loads; 1 or 2 = tensor-memory-accelerator copies
 * (cp.async.bulk.tensor) of each plane's E, H and code boxes into shared-memory rings.
 * With 4-row tiles, staging 1 sizes registers and shared memory for 3 CTAs per SM (rings
 * of 4 E and 2 H / code planes), staging 2 for 4 CTAs per SM (3 and 2 planes); 8-row
 * tiles run 2 CTAs per SM (3 and 2 planes) for either.  The copies run on coded
 * coefficients with Nx a multiple of 8 (and, in FP32, the 4-wide vector); elsewhere the
 * step keeps the loads.  l2_ahead (0..16): with the copies, the same boxes of that many
 * further planes are requested into L2 (cp.async.bulk.prefetch.tensor) ahead of the ring
 * loads, so those hit L2; 0 turns it off.  The rows and z ranges come from
 * fit_set_fused_shape.  Needs the fused
 * step enabled (FIT_ERR_STATE otherwise); returns FIT_ERR_ARG when the grid does not
 * qualify or the tensor maps cannot be encoded.
 * Same work as fit_set_fused_shape's kernel: the reference's _one_step
 * (wakis/solverFIT3D.py:504-525). */
FIT_API int fit_set_fused_staging(FitCtx *ctx, int32_t staging, int32_t l2_ahead);
/* Polls a kernel makes on a bounded wait for its bulk or tensor copies before it gives
 * up, records FIT_ERR_TIMEOUT (read by fit_check_error) and returns with its fields
 * unchanged from that point (staged passes, TMA-fed fused step).  Default 2^24; 0 gives up
 * at the first wait, which exercises the failure path without a fault.  After giving up a
 * kernel still waits (2^24 polls at most) for the copies it issued.  No counterpart in the
 * reference (its scipy step has no waits). */
FIT_API int fit_set_wait_limit(FitCtx *ctx, int64_t polls);
/* Times, beam off, on the context stream between CUDA events: reps fused steps from
 * (E, H) into the second buffers (ms_out[0]), and reps two-pass steps (H pass + E pass)
 * in place on copies of E and H in the second buffers (ms_out[1]); average milliseconds
 * per step.  E, H and J are not changed.  The solver's autotuner compares the two. */
FIT_API int fit_time_fused(FitCtx *ctx, int32_t reps, double *ms_out);

/* Benchmark support: launches the H pass reps times, then the elided-J E pass reps
 * times (advancing the fields), on the context's stream between CUDA events; ms_out
 * (host, 2 values) receives the average milliseconds per launch of each kernel. */
FIT_API int fit_time_kernels(FitCtx *ctx, int32_t reps, double *ms_out);

/* ---------------------------------------------------------------- serving pool
 * No counterpart in the reference: Wakis runs one solve per process, each wakesolve
 * (wakis/routines.py:231-485) stepping its own grid.  A pool advances many independent
 * FP32 contexts (grids of any size) together on one GPU: every step is three launches
 * that cover all member grids (wake taps + step counters, H pass, E pass), driven by a
 * device work table with one row per context and replayed from CUDA graphs in chunks of
 * chunk_steps steps.  A native driver thread runs the chunks (two in flight), retires
 * contexts whose steps are done and admits newly submitted ones at the next chunk, so
 * solves join and leave while others run (continuous batching).  Each context's fields,
 * wake sums and step counter evolve exactly as under fit_run: the per-cell arithmetic
 * is the same code.
 *
 * Memory admission: fit_pool_reserve / fit_pool_release keep a byte count against the
 * pool's budget; a caller reserves a solve's footprint before allocating it and
 * releases it after freeing it.  The pool never allocates field storage itself. */
typedef struct FitPool FitPool;

typedef struct FitPoolDone {
    int64_t tag;       /* the tag given to fit_pool_submit */
    int64_t steps;     /* steps taken */
    int32_t status;    /* FIT_OK, FIT_ERR_CANCELLED, or the error that stopped the pool */
    int32_t reserved;
    double t_submit_ms; /* host times in ms since fit_pool_create: submitted, */
    double t_start_ms;  /* first chunk containing the context launched, */
    double t_done_ms;   /* completion of its last chunk observed */
} FitPoolDone;

typedef struct FitPoolStats {
    int64_t chunks;         /* graph replays */
    int64_t cell_updates;   /* sum over contexts of N * steps taken */
    int64_t budget_bytes, reserved_bytes;
    int32_t active;         /* contexts in the work table or in flight */
    int32_t queued;         /* submitted, waiting for a table row */
    int32_t max_active;     /* most contexts stepped by one chunk */
    int32_t chunk_steps;
    int32_t variant[3];     /* pass-kernel variant (CTAs per SM) for vector widths 4, 2, 1 */
    int32_t grid[3];        /* persistent CTAs of the E pass for vector widths 4, 2, 1 */
    double busy_ms;         /* host time with at least one chunk in flight */
    int64_t fused_cell_updates;  /* the part of cell_updates taken by the fused kernel */
    int32_t fused_variant[3];    /* fused kernel variant (CTAs per SM) for vector widths 4, 2, 1 */
    int32_t fused_grid[3];       /* persistent CTAs of the fused kernel for vector widths 4, 2, 1 */
} FitPoolStats;

/* device: CUDA ordinal; budget_bytes > 0; chunk_steps in [1, 1024] (64 is a good
 * default); ctas_per_sm: persistent CTAs per SM of the pass kernels, 0 = as many as
 * the kernels' occupancy allows.  Starts the driver thread. */
FIT_API int fit_pool_create(int32_t device, int64_t budget_bytes, int32_t chunk_steps, int32_t ctas_per_sm,
                            FitPool **out);
/* Stops the driver after the chunks in flight; contexts still in the pool are
 * reported with status FIT_ERR_STATE and become usable again. */
FIT_API int fit_pool_destroy(FitPool *pool);
FIT_API int fit_pool_last_error(const FitPool *pool, char *buf, int64_t len);
/* FIT_OK, FIT_ERR_BUDGET (retry after a release), or FIT_ERR_ARG when bytes exceeds
 * the whole budget. */
FIT_API int fit_pool_reserve(FitPool *pool, int64_t bytes);
FIT_API int fit_pool_release(FitPool *pool, int64_t bytes);
/* Hands a ready FP32 context to the pool for steps n0 .. n0+nsteps-1, as fit_run(ctx,
 * n0, nsteps) would take them (elided J, beam from the v*t table, wake taps).  Work
 * queued on the context's streams before the call is ordered before its first pooled
 * step.  Until the pool reports the tag done, every other call on ctx fails with
 * FIT_ERR_STATE.  Contexts with a plane source or low-face ABC updates (emsolve
 * features) are rejected. */
FIT_API int fit_pool_submit(FitPool *pool, FitCtx *ctx, int64_t n0, int64_t nsteps, int64_t tag);
/* Copies up to max finished solves into out and returns how many (>= 0), waiting up to
 * wait_ms for the first one when none is ready and work is pending. */
FIT_API int fit_pool_poll(FitPool *pool, FitPoolDone *out, int32_t max, int32_t wait_ms);
/* Cancels the solve submitted with tag: a queued one is reported at once, a running one
 * gets no further chunks and is reported once the chunks in flight that step it have
 * completed, with status FIT_ERR_CANCELLED (unless those chunks took its last steps:
 * then it is reported finished, FIT_OK).  The other solves are not affected.  The
 * context is then usable again (its fields hold the steps taken).  FIT_ERR_ARG when no
 * queued or running solve has that tag.  No counterpart in the reference (one solve per
 * process). */
FIT_API int fit_pool_cancel(FitPool *pool, int64_t tag);
FIT_API int fit_pool_stats(FitPool *pool, FitPoolStats *out);
/* Chooses the pass kernels of one vector-width class (vec = 4, 2 or 1 cells per vector,
 * the widest that divides Nx): ctas_per_sm names the compiled variant by the CTAs per SM
 * its register budget is sized for (vec 4: 2 or 3, vec 2: 3 or 4, vec 1: 3 or 4; the
 * defaults are 3, 3 and 4).  Applies from the next chunk; graphs of the old variant are recaptured.
 * The serving layer's autotuner times the variants on the requests' own grids. */
FIT_API int fit_pool_tune(FitPool *pool, int32_t vec, int32_t ctas_per_sm);
/* Chooses the variant of the pooled fused step for one vector-width class (vec = 4, 2
 * or 1): ctas_per_sm names the register budget it was compiled for (vec 4: 2 or 3, vec
 * 2: 3 or 4, vec 1: 3 or 4; the defaults are 3, 3 and 4).  Applies from the next chunk.  No counterpart in the reference (one solve per
 * process there); the serving layer's autotuner calls it. */
FIT_API int fit_pool_tune_fused(FitPool *pool, int32_t vec, int32_t ctas_per_sm);

/* ---------------------------------------------------------------- field monitor
 * Running DFT of E at nf frequencies (FieldMonitor.update, wakis/field_monitors.py:59-101):
 * acc[f][c][n] += E_c[n] * phase[f], accumulated in FP64 complex, in the reference's
 * operation order.  acc (device) holds 3*nf*N complex128 values: component-major, then
 * frequency, then the flat cell index.  phase: host (re, im) pairs.  single != 0 rounds
 * each product to FP32 first, as numpy does for an FP32 field times a complex64 phase
 * (the phase of an FP32 time step); FP64 fields ignore it. */
/* One update from E (device, 3*N values of dtype), queued on stream (cudaStream_t; NULL =
 * legacy default stream); returns after the update completes. */
FIT_API int fit_monitor_update(const void *E, int32_t dtype, int64_t N, int32_t nf, const double *phase,
                               void *acc, int32_t single, void *stream);
/* Epilogue of the device step loop (fit_run; the wakesolve path with use_field_monitor):
 * after each step n0 <= n < n0 + nsteps, acc += E^(n+1) * phases[n - n0][f]; phases holds
 * nsteps*nf (re, im) pairs (copied to the device).  nf = 0 removes the epilogue. */
FIT_API int fit_set_monitor(FitCtx *ctx, int32_t nf, const double *phases, int64_t n0, int64_t nsteps,
                            void *acc, int32_t single);

/* Ez line history (the reference's Ez.h5 dump, wakis/routines.py:379-446): at every step
 * n0 <= n < n0 + nsteps, before the step (with the wake taps), E_z(lx[l], ly[l], k) of the
 * nlines (<= 9) lines for all k is written to hist[n - n0][l][k] (device, field dtype,
 * nsteps*nlines*Nz values).  nlines = 0 stops recording. */
FIT_API int fit_set_ez_record(FitCtx *ctx, void *hist, int32_t nlines, const int32_t *lx, const int32_t *ly,
                              int64_t n0, int64_t nsteps);
/* J_z line history of wakesolve(save_J=True) (wakis/routines.py:440-445), taken by the
 * step prologue like the Ez record: for steps n0 <= n < n0+nsteps, hist (device,
 * nsteps*nlines*Nz values of the field dtype) receives per line J_z after the beam
 * update and before the step -- the beam current on the beam's line, elsewhere
 * sigma_z*E_z of the previous step (a float64 product stored in the field dtype, as the
 * reference's J = sigma*E).  sigma_lines: host, nlines*Nz FP64 values of sigma_z on the
 * lines.  nlines = 0 turns the record off. */
FIT_API int fit_set_jz_record(FitCtx *ctx, void *hist, int32_t nlines, const int32_t *lx, const int32_t *ly,
                              int64_t n0, int64_t nsteps, const double *sigma_lines);

/* Library build information: sm architecture compiled for, and the kernel launch
 * counter (kernels issued since load), for bench accounting. */
FIT_API int fit_version(char *buf, int64_t len);
FIT_API int64_t fit_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* WAKIS_FIT_H */
