/*
 * bgk2d_gb300.h -- C ABI of libbgk2d_gb300.so, the GB300 (sm_103a) D2Q9 BGK time step.
 *
 * Drop-in boundary for the hot path of BGK2D.  The reference driver runs, once per step,
 *     call boundaries          (SRC/boundaries.F90:23-64  -> SRC/bcond.*.F90)
 *     call propagation         (SRC/propagation.F90:24-53 -> SRC/movef.F90)
 *     call collision(itime)    (SRC/collision.F90:24-55   -> SRC/col_MC.F90 / SRC/col.F90)
 * on populations held in `module storage` (SRC/storage.F90:86-112).  This library keeps the
 * populations resident in HBM behind an opaque handle; the three calls above map to
 * bgk_boundaries / bgk_propagation / bgk_collision (or one bgk_step), and the host-side
 * readers (diagno, draglift, probe/prof, vtk, save_raw) get their data from bgk_diagno,
 * bgk_draglift and bgk_download.
 *
 * Conventions
 *  - Every entry point returns an int status: BGK_OK (0) or a BGK_E_* code.  After an error
 *    the handle keeps its message (the most recent one); read it with bgk_last_error.  CUDA
 *    errors and kernel-side timeouts are sticky for the handle.
 *  - Host population arrays use the reference layout (SRC/alloca.F90:113-121): nine
 *    column-major arrays (0:lx+1+ipad, 0:ly+1+jpad), i fastest, leading dimension
 *    ld = lx+2+ipad, direction order 01,03,05,08,10,12,14,17,19 (SRC/bgk2d.F90:29-39),
 *    holding the deviations f_i - w_i (the reference's default "shifted" storage).
 *    The host element type is double for BGK_STORE_F64 and float otherwise.
 *  - One handle is used by one host thread at a time.
 */
#ifndef BGK2D_GB300_H
#define BGK2D_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BGK_ABI_VERSION 1

/* status codes */
#define BGK_OK 0
#define BGK_E_INVALID 1      /* bad argument or unsupported combination */
#define BGK_E_NOMEM 2        /* device allocation or admission failed */
#define BGK_E_CUDA 3         /* a CUDA call failed (sticky) */
#define BGK_E_UNSUPPORTED 4  /* feature not available for this case/scheme */
#define BGK_E_NUMERIC 5      /* NaN or Inf seen by a reduction */
#define BGK_E_CANCELLED 6    /* work cancelled by the host */
#define BGK_E_TIMEOUT 7      /* a bounded wait ran out */
#define BGK_E_NOTFOUND 8     /* unknown id */
#define BGK_E_TOOLARGE 9     /* size beyond a fixed limit of the entry point */

/* storage kind of the populations in HBM (SRC/precision.F90:13-47, `mystorage`) */
#define BGK_STORE_F32 0   /* SINGLE / MIXED2 */
#define BGK_STORE_F64 1   /* DOUBLE */
#define BGK_STORE_F16 2   /* 16-bit: (f_i - w_i) * s_i as IEEE half, s_i a power of two */
#define BGK_STORE_BF16 3  /* 16-bit: (f_i - w_i) * s_i as bfloat16 */

/* arithmetic kind of the collision (`mykind`) */
#define BGK_COMPUTE_F32 0
#define BGK_COMPUTE_F64 1

/* scheme */
#define BGK_SCHEME_PINGPONG 0  /* fused pull stream+collide, two buffers (SRC/col_MC.F90) */
#define BGK_SCHEME_AA 1        /* fused, one buffer, alternating even/odd access pattern */
#define BGK_SCHEME_ORIGINAL 2  /* two passes per step, as the ORIGINAL build: streaming (SRC/movef.F90)
                                  into the second buffer, then collision in place (SRC/col.F90);
                                  same results as ping-pong, twice its HBM traffic */

/* test case presets: the reference's compile-time case flags (SRC/Makefile:155-187) */
#define BGK_CASE_LDC 0     /* bcond_driven: walls + moving lid at y = ly+1 */
#define BGK_CASE_TGV 1     /* bcond_periodic */
#define BGK_CASE_POF 2     /* bcond_channel + body force fgrad */
#define BGK_CASE_VKS 3     /* bcond_inflow (+ obstacle, drag/lift) */
#define BGK_CASE_COU 4     /* bcond_couette */
#define BGK_CASE_BFS 5     /* bcond_step: backward-facing step, stepx = lx/20, stepy = ly/2
                              (SRC/input.F90:74-75); lx >= 40, ly >= 4.  The block x < stepx,
                              y < stepy is an obstacle: bgk_get_obs returns it */
#define BGK_CASE_MYV 6     /* -DMYVERSION: bcond_periodic with the CHANNEL body force fgrad
                              (SRC/boundaries.F90:46-48, SRC/build.bcond.F90:39-41) */
#define BGK_CASE_CUSTOM 9  /* faces[] and wall_u[] given explicitly */

/* face kinds for BGK_CASE_CUSTOM; faces are x_lo (i=0), x_hi (i=lx+1), y_lo, y_hi */
#define BGK_FACE_WALL 0         /* half-way bounce-back, optional wall velocity */
#define BGK_FACE_PERIODIC 1
#define BGK_FACE_INFLOW 2       /* x faces: equilibrium at rho=1, prescribed u (bcond.inflow.F90:101-113) */
#define BGK_FACE_OUTFLOW_EQ 3   /* x_hi: equilibrium at rho=1 and the local u (bcond.inflow.F90:80-99) */
#define BGK_FACE_OUTFLOW_ZG 4   /* x_hi: zero-gradient copy of column lx */

/* obstacle shapes (SRC/build.obs.F90) */
#define BGK_OBS_NONE 0
#define BGK_OBS_CIRCLE 1
#define BGK_OBS_SQUARE 2
#define BGK_OBS_HALF_CIRCLE 3
#define BGK_OBS_MASK 4      /* caller passes obs(1:lx,1:ly) */

/* initial states */
#define BGK_INIT_REST 0     /* init.F90 rest flow: all deviations zero */
#define BGK_INIT_TGV_REF 1  /* init.F90 periodic vortex, amplitude 0.1, rho = 1 */
#define BGK_INIT_TGV 2      /* vortex of amplitude tgv_u0 with rho = 1 - 3 u0^2/4 (cos 2kx + cos 2ky) */

typedef struct bgk_case_desc {
    int32_t lx, ly;           /* interior nodes (namelist lx, ly; SRC/input.F90:67-68) */
    int32_t ipad, jpad;       /* host array padding (namelist ipad, jpad) */
    int32_t storage;          /* BGK_STORE_* */
    int32_t compute;          /* BGK_COMPUTE_* */
    int32_t scheme;           /* BGK_SCHEME_* */
    int32_t tcase;            /* BGK_CASE_* */
    int32_t faces[4];         /* BGK_FACE_* for x_lo, x_hi, y_lo, y_hi (BGK_CASE_CUSTOM only) */
    double wall_u[4][2];      /* wall velocity (ux, uy) per face (BGK_CASE_CUSTOM only) */
    double svisc;             /* namelist svisc; omega = 2/(6 svisc + 1) (SRC/hencol.F90:30) */
    double u0;                /* namelist u0: lid speed (LDC/COU) or forcing velocity (POF) */
    double omega;             /* > 0 overrides the omega computed from svisc */
    double u_inflow;          /* peak inflow speed; <= 0 selects the reference's 0.1 */
    int32_t inflow_profile;   /* 0 uniform, 1 parabolic between half-way walls */
    int32_t obstacle;         /* BGK_OBS_* */
    int32_t radius;           /* namelist radius (SRC/input.F90:61) */
    int32_t obs_icoord;       /* obstacle centre; < 0 selects 2*lx/5 (SRC/build.obs.F90:174) */
    int32_t obs_jcoord;       /* < 0 selects ly/2 */
    const int32_t *obs_mask;  /* BGK_OBS_MASK: obs(1:lx,1:ly), column-major */
    int32_t init_v;           /* BGK_INIT_* applied by bgk_create */
    double tgv_u0;            /* amplitude for BGK_INIT_TGV */
    int32_t device;           /* CUDA device ordinal */
    int32_t les;              /* 1: Smagorinsky eddy viscosity in the collision (-DLES,
                                 SRC/col_MC.F90:178-248); such a handle steps with kernels of its
                                 own: bgk_tune picks the prefetch distance, and for 16-bit
                                 ping-pong also the kernel shape */
    double cte_s;             /* Smagorinsky constant cteS (namelist, SRC/input.F90:55; default 0.1) */
    int32_t trick1;           /* 1: the lid-cavity boundaries of the reference's -DTRICK1 build
                                 (SRC/bcond.driven.F90:43-81): its merged loop lets the side walls
                                 set the two upper corner ghosts, which then carry no lid term.
                                 BGK_CASE_LDC on a square box only (SRC/check_case.F90:173-178) */
    int32_t noshift;          /* 1: the reference's -DNOSHIFT build: the arrays hold the populations
                                 f themselves instead of the deviations f - w (SRC/col_MC.F90:70-75,
                                 SRC/init.F90:73-77, SRC/diagno.F90:42-46, ...).  FP32 and FP64
                                 storage only; ping-pong, AA and two-pass; not in batches */
    int32_t force_y;          /* 1: the reference's -DFORCING_Y build: the body force of
                                 BGK_CASE_POF / BGK_CASE_MYV / a forced BGK_CASE_CUSTOM acts along
                                 y (forcey = fgrad*rho, SRC/col_MC.F90:268-282); refused for the
                                 other cases */
    int32_t reserved[1];
} bgk_case_desc;

typedef struct bgk_handle bgk_handle;

/* Fill a descriptor with the reference defaults (LDC, FP32, ping-pong, radius 16). */
int bgk_default_desc(bgk_case_desc *desc);

/* Allocate the device state for one case and set it up like alloca + initialize
 * (SRC/alloca.F90, SRC/initialize.F90:70-128: build_bcond, build_obs, init, hencol).
 * Returns BGK_E_NOMEM when the populations do not fit in free HBM, and BGK_E_TOOLARGE when
 * ly > BGK_MAX_LY (the kernels put one lattice row, ghost rows included, per grid row). */
#define BGK_MAX_LY 65533
int bgk_create(const bgk_case_desc *desc, bgk_handle **out);
int bgk_destroy(bgk_handle *h);

/* Copy populations host -> device / device -> host (reference layout, see top).
 * pops[q] points at direction q's array; ld is its leading dimension in elements.  Page-locked
 * arrays (cudaHostAlloc, cudaHostRegister) are read or written in place by the transfer kernels,
 * the fastest and steadiest path; pageable arrays go through a device staging buffer.  Both
 * synchronise. */
int bgk_upload(bgk_handle *h, void *const pops[9], int64_t ld);
int bgk_download(bgk_handle *h, void *const pops[9], int64_t ld);

/* Upload `in`, run nsteps time steps, download into `out`: the same result, bit for bit, as
 * bgk_upload(in) + bgk_step(nsteps) + bgk_download(out), for a driver that keeps its populations
 * on the host between chunks of steps (the SRC/bgk2d.F90:92-113 loop with host arrays updated
 * at every diagnostic step).  `out` may be `in`.  With page-locked arrays, a ping-pong handle
 * and no periodic y face, backward-facing step, LES or two-pass form, the transfers and the
 * steps are pipelined: row bands go up, through the steps and back down in overlapping waves,
 * so a run of up to 32 steps costs about one round trip over the host link (longer runs pipeline
 * their first and last 16 steps).  Other cases run the three calls in sequence.  Synchronises. */
int bgk_advance_host(bgk_handle *h, void *const in[9], void *const out[9], int64_t ld, int32_t nsteps);

/* The reference's per-step call sequence.  bgk_boundaries and bgk_propagation record the
 * call order; the boundary rules and the streaming run inside the fused kernel launched by
 * bgk_collision (SRC/collision.F90:37-41 with FUSED).  Asynchronous. */
int bgk_boundaries(bgk_handle *h);
int bgk_propagation(bgk_handle *h);
int bgk_collision(bgk_handle *h, int32_t itime);

/* nsteps full time steps (boundaries + propagation + collision), replayed from CUDA graphs.
 * Asynchronous on the handle's stream. */
int bgk_step(bgk_handle *h, int32_t nsteps);
/* Same, bracketed by CUDA events on the handle's stream; *ms = device time (synchronises). */
int bgk_step_timed(bgk_handle *h, int32_t nsteps, float *ms);
int bgk_sync(bgk_handle *h);

/* Reductions over the interior (synchronise).
 * diagno (SRC/diagno.F90:63-101): out = <u>, <v>, <rho>, <|u|^2>.  mode BGK_DIAGNO_ALL sums in FP64
 * over all cells, BGK_DIAGNO_FLUID skips obstacle cells, BGK_DIAGNO_REFERENCE sums in the compute
 * kind in the reference's sequential j/i order and divides as it does, so the means equal the
 * values the reference writes to diagno.dat (one block on the GPU: slower, for output files). */
#define BGK_DIAGNO_ALL 0
#define BGK_DIAGNO_FLUID 1
#define BGK_DIAGNO_REFERENCE 2
int bgk_diagno(bgk_handle *h, int32_t fluid_only, double out[4]);
/* momentum-exchange drag/lift (SRC/draglift.F90:41-100): out = Fx*norm, Fy*norm */
int bgk_draglift(bgk_handle *h, double out[2]);
/* the same in the reference's own arithmetic and order (compute-kind sums over the box, serial
 * j/i, x then y; SRC/draglift.F90:41-100), the values it writes to drag.lift; box cells outside
 * the interior are skipped */
int bgk_draglift_reference(bgk_handle *h, double out[2]);
/* steady-state residual: ||u - u_prev||_2 / ||u||_2 since the previous call (first call: 1) */
int bgk_residual(bgk_handle *h, double *out);
/* macroscopic fields rho, u, v of the interior to host arrays of lx*ly doubles, i fastest */
int bgk_fields(bgk_handle *h, double *rho, double *u, double *v);
/* obstacle mask obs(1:lx,1:ly) and imin,imax,jmin,jmax,nobs (SRC/build.obs.F90) */
int bgk_get_obs(bgk_handle *h, int32_t *mask, int32_t bbox[5]);
/* The fields the reference's VTK writers compute on the host after a device-to-host update
 * (SRC/vtk_xy.binary.F90:75-140, SRC/vtk_om.binary.F90:61-155), computed on the device in their
 * single-precision arithmetic, so that 5 float fields cross the bus instead of 9 populations:
 * u/rho, w/rho, rho over the interior (lx*ly each, x fastest), vorticity and stream function over
 * x = 2..lx-1, y = 2..ly-1 ((lx-2)*(ly-2) each).  The stream function integrates from row 1: the
 * reference starts at ghost row 0, whose values the fused step keeps nowhere (in the reference's
 * FUSED build that term reads the ghost row of the buffer written two steps earlier).  Any
 * output pointer may be NULL. */
int bgk_vtk_fields(bgk_handle *h, float *u, float *w, float *rho, float *vort, float *stream);
/* The profile readers the reference runs on the host after a device-to-host update at each
 * diagnostic stop (SRC/diagnostic.F90:70-82), computed on the device with their arithmetic, so that
 * profiles cross the bus instead of 9 populations: the stored values summed in the storage kind as
 * they lie in the arrays, cte1 added and the quotients taken in the compute kind (FP64 under
 * MIXED2); probe in compute-kind temporaries.  The doubles hold compute-kind values exactly.
 *   bgk_prof_i: u, v, den along row jcoord, i = 1..lx (SRC/prof_i.F90:47-62; lx values each)
 *   bgk_prof_j: u, v, den along column icoord, j = 1..ly (SRC/prof_j.F90:47-67; ly values each)
 *   bgk_varm:   row means of u, w, den over i = 1..lx for j = 1..ly (SRC/varm.F90:49-88, u_med.dat)
 *   bgk_probe:  u, v, rho at (i0, j0) (SRC/probe.F90:46-62)
 * Coordinates outside 1..lx / 1..ly return BGK_E_INVALID. */
int bgk_prof_i(bgk_handle *h, int32_t jcoord, double *u, double *v, double *den);
int bgk_prof_j(bgk_handle *h, int32_t icoord, double *u, double *v, double *den);
int bgk_varm(bgk_handle *h, double *u, double *w, double *den);
int bgk_probe(bgk_handle *h, int32_t i0, int32_t j0, double out[3]);
/* omega, fgrad, u00, u0 after build_bcond + hencol, and the step counter */
int bgk_get_scalars(bgk_handle *h, double out[4], int64_t *itime);

/* thread-block tile shape of the step kernels (no reference counterpart):
 *   0 = 32x4 threads, 1 = 64x2, 2 = 128x1, 3 = 128x2, each thread updating one 16-byte vector
 *   of cells per plane; 4 = 32x4 and 5 = 128x1 with half a vector (8 bytes) per thread.  Ping-pong only: 6, 7, 8 stage the source rows in shared memory with bulk
 *   async copies (128 threads and 3 rows in flight, 128 and 4, 256 and 3; 8 bytes per thread);
 *   such a step reports BGK_E_TIMEOUT at the next synchronisation if a copy never completed.
 *   Results do not depend on the choice, with one exception: AA with 16-bit storage rounds
 *   each value that crosses a warp edge on its own, so shapes 0-3 and shapes 4-5 give slightly
 *   different populations (identical within each group). */
int bgk_set_tile(bgk_handle *h, int32_t tile_cfg);
/* configurations 0-5 (ping-pong and AA): each block first asks for an L2 prefetch (bulk, no
 * registers) of the source rows of the block `blocks_ahead` places further on in launch order;
 * 0 = off (no reference counterpart).  Results do not depend on it. */
int bgk_set_prefetch(bgk_handle *h, int32_t blocks_ahead);
int bgk_get_prefetch(bgk_handle *h, int32_t *blocks_ahead);
/* time `trial_steps` real steps per tile shape and prefetch distance (the state advances) and
 * keep the fastest.  AA with 16-bit storage tries shapes 4 and 5 only, so the populations of a
 * tuned run do not depend on which shape wins. */
int bgk_tune(bgk_handle *h, int32_t trial_steps, int32_t *tile_cfg, int32_t *steps_run);

/* bytes of HBM the handle holds, and the algorithmic bytes moved per lattice update */
int bgk_footprint(bgk_handle *h, int64_t *device_bytes, int32_t *bytes_per_cell);
/* number of kernels this library launched on the handle so far */
int bgk_launch_count(bgk_handle *h, int64_t *launches);

/* Measured FP64 instruction rates of a device: out = DFMA, DADD and DMUL thread operations per
 * second, from independent chains of each on every SM (CUDA events, best of five).  GB300 runs
 * FP64 at a small fraction of its FP32 rate, so this, not HBM, bounds the DOUBLE and MIXED2
 * steps.  No counterpart in the reference (a measurement helper).  Synchronises. */
int bgk_peak_fp64(int32_t device, double out[3]);
int bgk_last_error(bgk_handle *h, char *buf, size_t len);
const char *bgk_version(void);

/* diagno sums without any allocation.  No counterpart in the reference.
 * For callers that cannot let the library allocate device memory: a Fortran OpenACC or
 * OpenMP-offload build whose populations live in data regions owned by the compiler's runtime,
 * or a program running under a fixed device-memory budget.  The caller passes device pointers
 * to its own nine population arrays (reference layout and direction order, leading dimension
 * ld >= lx+2, deviations f - w, float for BGK_STORE_F32 or double for BGK_STORE_F64) and a
 * host array for out = <u>, <v>, <rho>, <|u|^2> (SRC/diagno.F90 per-cell arithmetic, FP64
 * sums).  The partial sums go to one static device array of 128 KiB that every GPU loading the
 * library holds until exit; lx*ly may be at most 16,777,216 (4096^2), larger domains return
 * BGK_E_TOOLARGE.  Nothing is allocated: no cudaMalloc/cudaFree, no pools.  Every call looks
 * up the array's device address in the current context (cudaGetSymbolAddress); the first call
 * on a device also loads the library's device code there, so make that first call before any
 * stream capture.  Runs on the legacy default stream and returns when the means are on the
 * host; the caller orders its own writes to the arrays before the call.  All calls share the
 * array, so calls from several host threads are serialised by a process-wide lock.  When a
 * sum is not finite the call returns BGK_E_NUMERIC and out holds the non-finite means. */
int bgk_diagno_noalloc(const void *const pops[9], int64_t ld, int32_t lx, int32_t ly, int32_t storage,
                       double out[4]);

/* ---------------------------------------------------------------------------------------------
 * Batches: many independent ping-pong cases of one (storage, compute) kind advanced together,
 * one persistent work-list launch per time step, replayed from CUDA graphs.  No reference
 * counterpart (the reference runs one domain per process, SRC/bgk2d.F90:92-113).  While a
 * handle is attached, bgk_step/bgk_collision on it return BGK_E_INVALID; every other handle
 * call works and waits for the batch's last step.
 * ------------------------------------------------------------------------------------------- */
typedef struct bgk_batch bgk_batch;
int bgk_batch_create(int32_t storage, int32_t compute, int32_t device, bgk_batch **out);
int bgk_batch_destroy(bgk_batch *b);
int bgk_batch_add(bgk_batch *b, bgk_handle *h);
int bgk_batch_remove(bgk_batch *b, bgk_handle *h);
int bgk_batch_size(bgk_batch *b, int32_t *members, int64_t *cells);
int bgk_batch_step(bgk_batch *b, int32_t nsteps);
int bgk_batch_step_timed(bgk_batch *b, int32_t nsteps, float *ms);
int bgk_batch_sync(bgk_batch *b);
/* tile shape (as bgk_set_tile), persistent blocks per SM (0: one block per work-list tile,
 * no persistent loop), steps per CUDA graph (even) */
int bgk_batch_set_config(bgk_batch *b, int32_t tile_cfg, int32_t blocks_per_sm, int32_t graph_steps);
/* one block per tile (blocks_per_sm = 0): L2 prefetch of the work-list entry `tiles_ahead` places
 * further on (0 = off); the autotuner sets it */
int bgk_batch_set_prefetch(bgk_batch *b, int32_t tiles_ahead);
int bgk_batch_get_config(bgk_batch *b, int32_t out[3]);
/* autotuner: times real steps over tile shapes, grid sizes and graph lengths; keeps the best */
int bgk_batch_tune(bgk_batch *b, int32_t trial_steps, int32_t *steps_run);
int bgk_batch_launch_count(bgk_batch *b, int64_t *launches);

/* ---------------------------------------------------------------------------------------------
 * Serving loop: solves submitted as they arrive are admitted against free HBM and a slot
 * limit, keep their populations resident between step chunks, are advanced together in the
 * batched kernel (one batch per storage kind, batches on separate streams), and return their
 * diagnostics and fields on completion.  A request stops at max_steps, or earlier when its
 * residual (checked every check_every of its own steps) drops below tol.  No reference
 * counterpart.  All calls are thread-safe.
 * ------------------------------------------------------------------------------------------- */
#define BGK_REQ_LDC 0       /* lid-driven cavity n x n, lid speed u, nu = u n / re */
#define BGK_REQ_CYLINDER 1  /* channel 16D x 4D, cylinder D = n at (4D, 2D+1), parabolic inflow of
                               peak u, zero-gradient outflow, walls; nu = u D / re; drag/lift */
#define BGK_REQ_TGV 2       /* periodic Taylor-Green n x n, amplitude u, nu = u n / re */

typedef struct bgk_request {
    int32_t kind;        /* BGK_REQ_* */
    int32_t n;           /* cavity / vortex edge, or cylinder diameter */
    double re;           /* Reynolds number */
    double u;            /* lid speed, inflow peak or vortex amplitude */
    int32_t storage;     /* BGK_STORE_F32 / F64 / F16 / BF16 */
    int32_t max_steps;   /* step budget */
    double tol;          /* residual tolerance; <= 0 runs max_steps */
    int32_t check_every; /* steps between residual checks (> 0) */
    int32_t keep_fields; /* 1: keep rho, u, v for bgk_server_fields */
} bgk_request;

typedef struct bgk_result {
    int64_t id;
    int32_t status;       /* BGK_OK; BGK_E_NUMERIC when a residual or the final means are not
                             finite; BGK_E_NOMEM when the request can never fit the budget; the
                             status of a failed bgk_create, or of a failed step of its batch */
    int32_t steps;
    int32_t lx, ly;
    double residual;      /* last residual (0 when never checked) */
    double diagno[4];     /* <u>, <v>, <rho>, <|u|^2> at completion */
    double draglift[2];   /* cylinder only */
    double t_submit, t_admit, t_done;  /* seconds since server start */
} bgk_result;

typedef struct bgk_server_config {
    int32_t device;
    int32_t max_slots;       /* concurrently resident requests */
    int64_t hbm_budget;      /* bytes the server may hold; <= 0: free HBM minus 4 GiB */
    int32_t chunk_steps;     /* steps per scheduling round (upper bound) */
    int32_t tile_cfg;        /* batch tile shape (bgk_set_tile numbering, 0..5); < 0 selects 64x2
                                (FP32/FP64) or 128x1 with 8 bytes per thread (16-bit) */
} bgk_server_config;

typedef struct bgk_server_stats {
    int64_t submitted, admitted, completed, failed;
    int64_t cell_updates;     /* lattice updates of all requests */
    double busy_s;            /* wall time spent in step rounds */
    double wall_s;            /* first admission to last completion */
    double glups;             /* cell_updates / wall_s / 1e9 */
    double p50_s, p99_s;      /* latency (t_done - t_submit) percentiles */
    double mean_queue_s;      /* mean t_admit - t_submit */
    int32_t peak_resident;
    int64_t launches;         /* kernels launched by the server */
    int64_t rounds;           /* scheduling rounds */
    double mean_round_steps;  /* steps per round */
} bgk_server_stats;

typedef struct bgk_server bgk_server;
int bgk_server_create(const bgk_server_config *cfg, bgk_server **out);
int bgk_server_destroy(bgk_server *s);
int bgk_server_submit(bgk_server *s, const bgk_request *req, int64_t *id);
/* move up to max finished results into out (oldest first); *n = how many */
int bgk_server_poll(bgk_server *s, bgk_result *out, int32_t max, int32_t *n);
/* block until every submitted request finished or timeout_s elapsed (BGK_E_TIMEOUT) */
int bgk_server_drain(bgk_server *s, double timeout_s);
/* fields of a finished request that asked for them: lx*ly doubles each, i fastest, into arrays
 * of `capacity` doubles each.  BGK_E_INVALID when capacity < lx*ly (the fields stay kept);
 * BGK_E_NOTFOUND when the request kept none or they were already taken. */
int bgk_server_fields(bgk_server *s, int64_t id, double *rho, double *u, double *v, int64_t capacity);
int bgk_server_get_stats(bgk_server *s, bgk_server_stats *out);

#ifdef __cplusplus
}
#endif
#endif
