/*
 * ufo_gb300.h -- C ABI of the GB300 tracking library (libufo_gb300.so).
 *
 * The reference (bellaz89/ufo) is pure Python: for every simulation object it
 * generates an OpenCL C kernel with the lattice pasted in as literals, builds
 * it with pyopencl and, in run(), copies the parameter pool to the device,
 * launches the kernel and copies the result back.  This library replaces that
 * generated kernel and its buffer plumbing with precompiled sm_103a kernels
 * that interpret a lattice opcode table (built by ufo_gb300/compiler.py).
 * Each entry point names the reference code it replaces.
 *
 * Conventions: every call returns 0 on success or a negative UFO_E* code;
 * ufo_last_error() then returns a message (thread-local).  Host pointers are
 * owned by the caller and only accessed during the call.  Calls on one
 * context are not thread-safe (the reference's command queue was not either).
 * Arithmetic is IEEE FP64.
 */
#ifndef UFO_GB300_H
#define UFO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UFO_OK 0
#define UFO_E_ARG (-1)       /* invalid argument (sizes, NULL, opcode table) */
#define UFO_E_CUDA (-2)      /* CUDA runtime error */
#define UFO_E_NOMEM (-3)     /* device allocation failed */

/* track modes: loss test at the end of each turn */
#define UFO_MODE_TRACK 0     /* isnan(x)                        ufo/track.py:107-108 */
#define UFO_MODE_SA 1        /* |x|>1 || |y|>1 || isnan(x)      ufo/sa.py:118-119    */

/* track flags */
#define UFO_TRACK_FMA 1      /* fused multiply-add arithmetic (tolerance parity) */
#define UFO_TRACK_FIVED 2    /* do not write z, dp into tracks (ufo/track.py:62-65) */
#define UFO_TRACK_PLAIN 4    /* one thread per particle, no lane refill */
#define UFO_TRACK_COMPACT 8  /* persistent CTAs (one per SM, warps_per_sm warps, at most
                                16) that pack survivors into full warps once every particle
                                is handed out and even out their particle counts through
                                the context's particle pool (ufo_track_noalloc: packing
                                within each CTA only); PLAIN takes precedence.  Every
                                kernel gives the same results bit for bit. */

#define UFO_OP_WORDS 8

typedef struct ufo_ctx ufo_ctx;    /* device, stream, scratch            */
typedef struct ufo_prog ufo_prog;  /* a compiled line resident on device */

/* Last error message of the calling thread ("" if none). */
const char *ufo_last_error(void);

/* Number of CUDA devices; replaces ufo/cl_utils.py:12-28 (list_devices). */
int ufo_device_count(int *count);

/* Create a context on `device` with its own stream; replaces the OpenCL
 * context + command queue of ufo/cl_utils.py:30-33 and ufo/track.py:44-45.
 * Holds the work counters and the compacting kernel's particle pool (80 bytes
 * per lane of the largest compacting grid: SMs x 512, 6.2 MB on 152 SMs).
 * Launches through one context share them: serialise them on one stream. */
int ufo_ctx_create(int device, ufo_ctx **out);
void ufo_ctx_destroy(ufo_ctx *ctx);

/* Upload a compiled line: `ops` int32[n_ops][8], `table` f64[n_seeds][stride],
 * `n_dumps` observation points per turn.  Replaces the kernel build of
 * ufo/track.py:84-118 (cl.Program(...).build). */
int ufo_prog_create(ufo_ctx *ctx, const int32_t *ops, int n_ops, const double *table,
                    int64_t stride, int n_seeds, int n_dumps, ufo_prog **out);
/* Replace the per-seed constants (same stride); new parameter values between
 * runs, the role of the reference's `.parameters` buffer for lattice values.
 * Every row's aperture and dynamic-kick programs are checked as at creation. */
int ufo_prog_set_table(ufo_prog *prog, const double *table, int n_seeds);
void ufo_prog_destroy(ufo_prog *prog);

/*
 * Track particles (host buffers, synchronous).  Replaces Track.run
 * (ufo/track.py:125-139) + its kernel (:84-114) and StableAperture.run
 * (ufo/sa.py:131-145) + its kernel (:93-126).
 *   coords  f64[n][6]  x, px, y, py, z, dp at turn 0
 *   seed    i32[n]     constant-table row of each particle, or NULL (row 0)
 *   pturns  i32[n]     turns of each particle, or NULL (`turns` for all)
 *   mode    UFO_MODE_TRACK / UFO_MODE_SA;  flags  UFO_TRACK_*
 *   slots   observation slots per particle in `tracks` (count*turns/every);
 *           0 disables tracks
 *   every   observe on turns t with (t+1) % every == 0 (1 = every turn)
 *   tracks  f64[n][slots][6] or NULL; unwritten slots are 0
 *   lost    u32[n] or NULL: turn at whose end the particle was lost, else its
 *           number of turns
 *   final   f64[n][6] or NULL: coordinates after the last tracked turn
 */
int ufo_track(ufo_ctx *ctx, const ufo_prog *prog, const double *coords, const int32_t *seed,
              const int32_t *pturns, int64_t n, int turns, int mode, int flags, int64_t slots,
              int every, double *tracks, uint32_t *lost, double *final_state);

/* Same, with device pointers, enqueued on `stream` (NULL: the context's
 * stream) without synchronising; device buffers are the caller's. */
int ufo_track_device(ufo_ctx *ctx, const ufo_prog *prog, const double *d_coords,
                     const int32_t *d_seed, const int32_t *d_pturns, int64_t n, int turns,
                     int mode, int flags, int64_t slots, int every, double *d_tracks,
                     uint32_t *d_lost, double *d_final, void *stream);

/* Largest opcode table ufo_track_noalloc accepts. */
#define UFO_NOALLOC_MAX_OPS 8192

/*
 * Allocation-free tracking.  No counterpart in the reference (which always
 * creates its own OpenCL buffers); it exists for callers that cannot call
 * cudaMalloc -- programs whose GPU memory belongs to another allocator (a
 * framework's memory pool or a fixed arena) or that must not allocate while
 * running, such as an online model in an accelerator control loop, where an
 * allocation could stall or fail mid-operation.  Needs no context or program
 * object: pass the host opcode table (`ops`, int32[n_ops][8], at most
 * UFO_NOALLOC_MAX_OPS rows, else UFO_E_ARG) and device pointers for the
 * per-seed constants (`d_table`, f64[n_seeds][stride]), the coordinates and
 * the outputs; the other arguments mean what they mean in ufo_track_device.
 * Works on the current device and enqueues on `stream` (NULL: the legacy
 * default stream) without synchronising.
 * It calls no cudaMalloc, cudaFree or other allocating routine.  Its scratch
 * (the staged opcode table and the work counter) is a static device array of
 * 256.25 KiB that every GPU loading this library holds until exit.  Every call
 * shares that array: calls that overlap on the GPU race (serialise them on one
 * stream); each call clears the counter it needs.  The first call on a device
 * sets up that device (resolves the array's address, uploads constant tables);
 * make that first call before any stream capture.  That set-up is not redone:
 * cudaDeviceReset after the first call is not supported.
 * `ops` is copied with cudaMemcpyAsync on `stream`: from pageable memory the
 * call returns after the copy has taken it; from pinned (page-locked) memory
 * the copy runs later, so keep `ops` unchanged until the stream has passed the
 * call.  Checks: op shapes, constant offsets against `stride` and observation
 * indices against `n_dumps` (UFO_E_ARG before any GPU work).  The constants are
 * on the device, so the aperture and dynamic-kick expression programs inside
 * `d_table` are NOT checked as ufo_prog_create checks them; pass tables made
 * by the lattice compiler (ufo_gb300/compiler.py).  A malformed program there
 * stays in bounds (the kernels bound their expression stacks) but gives a NaN
 * coefficient or a wrong loss test instead of an error.
 * With UFO_TRACK_COMPACT the CTAs pack their survivors but exchange none: the
 * particle pool they would exchange through belongs to a context.
 */
int ufo_track_noalloc(const int32_t *ops, int n_ops, const double *d_table, int64_t stride,
                      int n_seeds, int n_dumps, const double *d_coords, const int32_t *d_seed,
                      const int32_t *d_pturns, int64_t n, int turns, int mode, int flags,
                      int64_t slots, int every, double *d_tracks, uint32_t *d_lost,
                      double *d_final, void *stream);

/* Closed orbits by the reference's Nelder-Mead search (ufo/co.py:18-124, the
 * ClosedOrbit kernel :146-250): `iterations` steps on the squared one-turn
 * residual of (x, px, y, py) at z = 0, dp = 0, oodppo = 1, from the simplex
 * {v, v + 1e-4 e_j}, in the reference's operation order with the strict
 * one-turn map, so the orbits equal the reference's.  Host buffers:
 *   start  f64[n][4] first vertex of each orbit (the reference's x/px/y/py
 *          parameters, zero where absent)
 *   seed   i32[n] constant-table row of each orbit, or NULL (row 0)
 *   orbits f64[n][4] out: the best vertex after `iterations` steps */
int ufo_closed_orbit(ufo_ctx *ctx, const ufo_prog *prog, const double *start,
                     const int32_t *seed, int64_t n, int iterations, double *orbits);

/* Resident warps per SM of the persistent grid (default 16); set by the
 * autotuner (ufo_gb300/batch.py: autotune).  No reference counterpart. */
int ufo_ctx_set_tuning(ufo_ctx *ctx, int warps_per_sm);

/* One tracking launch (work-counter reset + persistent kernel over all
 * particles of all seeds) captured into a CUDA graph and replayed on the same
 * device buffers: the batched-seed path (many lattice variants with uneven
 * particle and turn counts in one launch).  Replaces the reference's idiom of
 * per-particle parameter rows in one NDRange (HOWTO.md:21, ufo/track.py:110). */
typedef struct ufo_graph ufo_graph;
int ufo_graph_create(ufo_ctx *ctx, const ufo_prog *prog, const double *d_coords,
                     const int32_t *d_seed, const int32_t *d_pturns, int64_t n, int turns,
                     int mode, int flags, int64_t slots, int every, double *d_tracks,
                     uint32_t *d_lost, double *d_final, ufo_graph **out);
int ufo_graph_launch(ufo_graph *graph, void *stream);
void ufo_graph_destroy(ufo_graph *graph);

/*
 * Tangent map and adjoint of the one-turn map (no reference counterpart: the
 * reference differentiates only by finite differences of tunes in dp,
 * tests/optics3.py:13-23).  Device pointers throughout, asynchronous on
 * `stream`; 0 on success, -1 bad argument, -2 launch error.  `ops` is the
 * differentiator's opcode list int32[n_ops][8] and `tab` its constants (built
 * by ufo_gb300/diff.py), one row of `tab_stride` constants per seed, `seed`
 * int32[J] the row of each job (NULL: row 0); one job per thread.
 *   ufo_diff_forward: z0 f64[J][4], o f64[J] (1/(1+dp)) -> zT f64[J][20]
 *     (state and, with `tangent`, the 4x4 Jacobian), checkpoints
 *     f64[turns/ck+1][20][J] every `ck` turns (NULL: none)
 *   ufo_diff_reverse: the checkpoints of the forward call, output cotangents
 *     zbar f64[J][4] (and Tbar f64[J][16]) -> zbar0 f64[J][4], parameter
 *     cotangents pbar f64[n_params][J].  Scratch tape
 *     f64[tape_segments * ck][ceil(J/32)][kicks_per_turn][nf][32] (warp-blocked,
 *     16-byte aligned): with `tangent` nf = 10 and
 *     one segment is taped at a time (tape_segments = 1 suffices); without it
 *     nf = 4 and tape_segments checkpoint segments are re-tracked in parallel
 *     (G x J jobs) before they are reversed, so a larger tape shortens the pass.
 */
int ufo_diff_forward(const int32_t *ops, int n_ops, const double *tab, int64_t tab_stride,
                     const int32_t *seed, int n_params, int kicks_per_turn, int n_jobs,
                     const double *z0, const double *o, int turns, int ck, int tangent,
                     double *ckpt, double *zT, void *stream);
int ufo_diff_reverse(const int32_t *ops, int n_ops, const double *tab, int64_t tab_stride,
                     const int32_t *seed, int n_params, int kicks_per_turn, int n_jobs,
                     const double *o, int turns, int ck, int tangent, const double *ckpt,
                     const double *zbar, const double *Tbar, double *tape, int tape_segments,
                     double *zbar0, double *pbar, void *stream);

/* Kernel launches issued by this library since the context was created.
 * Diagnostic; no reference counterpart. */
int ufo_launch_count(ufo_ctx *ctx, int64_t *count);

/* Measured FP64 FMA throughput of the device in GFLOP/s (2 flops per DFMA),
 * best of 3 timed launches of an independent-chain DFMA kernel.  Diagnostic
 * (the roofline denominator of the benchmark); no reference counterpart. */
int ufo_fp64_peak(ufo_ctx *ctx, double *gflops);

/* FP64-pipe probe (no reference counterpart): one-warp blocks, `warps_per_sm`
 * per SM, `chains` (1, 2, 4 or 8) independent DFMA chains per thread, only the
 * first `lanes` lanes of each warp active; *gflops counts the active lanes'
 * flops (2 per DFMA).  Shows what latency, occupancy and inactive lanes cost. */
int ufo_fp64_probe(ufo_ctx *ctx, int warps_per_sm, int chains, int lanes, double *gflops);

#ifdef __cplusplus
}
#endif
#endif
