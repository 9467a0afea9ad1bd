/*
 * glemur.h -- C-ABI of the GB300-native magneto-frictional relaxation library.
 *
 * The reference (SimonCan/glemur) exposes no library API: its hot path is the
 * kernel sequence that src/main.cu:259-384 drives, configured by the Fortran
 * namelist src/readNamelist.f90 into struct Parameters (src/global.h:44-108).
 * Each entry point below replaces one piece of that sequence; the comment on
 * each cites the reference code it stands in for.
 *
 * Conventions
 *   - Host arrays crossing this ABI use the reference layout: AoS, component
 *     fastest, one ghost layer, index l + 3*(i + (nx+2)*(j + (ny+2)*k)) for
 *     ghosted fields (xb, B0, B) and l + 3*(i + nx*(j + ny*k)) for the
 *     inner-only current J (src/rungeKutta.cu:50-51, src/current.cu:401).
 *     detJac is ghosted and scalar.  Element type is float when
 *     params.precision == 32 and double when it is 64 (the reference REAL,
 *     src/global.h:20-35).
 *   - Ownership: host buffers stay with the caller; device buffers belong to
 *     the handle.  No entry point calls exit().
 *   - Threading: one handle per host thread; all device work runs on the
 *     handle's stream (gm_set_stream), never on the legacy default stream.
 *   - Errors: every call returns GM_OK (0) or a negative GM_E* code;
 *     gm_last_error() gives a message for the calling thread.
 */
#ifndef GLEMUR_H_
#define GLEMUR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GM_STR_LEN 30
#define GM_MAX_BLOBS 10

/* Status codes. */
#define GM_OK            0
#define GM_EPARAM       -1   /* invalid parameter or argument                  */
#define GM_EALLOC       -2   /* device or host allocation failed              */
#define GM_ECUDA        -3   /* a CUDA runtime call failed                    */
#define GM_ENAN         -4   /* NaN/Inf seen in a stage increment             */
#define GM_EDETJAC      -5   /* a cell with detJac <= 0 was seen               */
#define GM_EDTMIN       -6   /* dt fell to dtMin (reference stop rule)         */
#define GM_ETIMEOUT     -7   /* a bounded device wait ran out                  */
#define GM_ENOTREADY    -8   /* call order violated (e.g. step before upload)  */
#define GM_EIO          -9   /* file input/output error (driver helpers)       */

/* Device status bits (gm_state.status). */
#define GM_ST_NAN        1u
#define GM_ST_DETJAC     2u
#define GM_ST_DTMIN      4u
#define GM_ST_DONE       8u
#define GM_ST_TIMEOUT   16u   /* a bounded wait on an asynchronous copy ran out */
#define GM_ST_ALIGN     32u   /* a copy was skipped: its shared-memory or tensor-map alignment check failed */
#define GM_ST_EVENT     64u   /* gm_run_events stopped after an accepted step with output due */

/* Output events of an accepted step (gm_state.event), the triggers of
 * src/main.cu:355-377 evaluated on the device after the dt update. */
#define GM_EV_TS         1    /* timeIndex % nTs == 0: reductions + time-series row */
#define GM_EV_DUMP       2    /* ceil((t-dt)/dtDump) != ceil(t/dtDump): data/dump<n>.vtk */
#define GM_EV_SAVE       4    /* ceil((t-dt)/dtSave) != ceil(t/dtSave): data/save.vtk */
#define GM_EV_LAST       8    /* last accepted step of the run (timeIndex == nCycle-1): data/save.vtk */

/*
 * Run parameters.  Mirrors struct Parameters (src/global.h:44-108) field by
 * field and in the same order, with REAL widened to double and bool stored
 * as int32_t.  Real values must already be rounded to the run precision
 * (the namelist reader in this library does that, exactly as the Fortran
 * reader reads into REAL, src/readNamelist.f90:173-255).  Strings are blank
 * padded to 29 characters plus a NUL, as copyString produces them
 * (src/readNamelist.f90:267-283).  Fields after the reference's last field
 * are extensions with no counterpart in the reference.
 */
typedef struct gm_params {
    int32_t nx, ny, nz;
    double  Lx, Ly, Lz;
    double  Ox, Oy, Oz;
    double  dx, dy, dz;
    double  dx1, dy1, dz1;
    char    bInit[GM_STR_LEN];
    char    uInit[GM_STR_LEN];
    double  ampl;
    double  phi1, phi2;
    double  L1, L2;
    double  ar, az;
    int32_t nBlobs;
    double  width;
    double  minor, major;
    double  stretch;
    double  bGround;
    double  blobXc[GM_MAX_BLOBS], blobYc[GM_MAX_BLOBS], blobZc[GM_MAX_BLOBS];
    double  blobZl[GM_MAX_BLOBS], blobTwist[GM_MAX_BLOBS], blobScale[GM_MAX_BLOBS];
    char    initDist[GM_STR_LEN];
    int32_t initDistCode;
    double  initShearA, initShearB, initShearK;
    double  pert;
    double  twist;
    int32_t fRestart;
    int32_t nCycle;
    double  dt0, dtMin, maxError;
    int32_t zUpdate, inertia, pressure;
    double  nu, beta;
    int32_t jxbAver;
    double  jxbAverWeight;
    int32_t xPeri, yPeri, zPeri;
    int32_t epsilonProf;
    char    jMethod[GM_STR_LEN];
    char    pMethod[GM_STR_LEN];
    int32_t nTs;
    double  dtDump, dtSave;
    int32_t dumpJ, dumpDetJac, dumpCellVol, dumpConvexity, dumpWedgeMin;
    int32_t redB2, redB2f, redBMax, redJMax, redJxB_B2Max, redEpsilonStar;
    int32_t redErrB_1ez, redErrXb_XbAn, redConvex, redWedgeMin, redU2, redUMax;
    /* ---- extensions ---- */
    int32_t precision;   /* 32: float storage, 64: double storage (PRECISION, src/Makefile:11) */
    int32_t errMode;     /* 0: error norm |x_new - x*| in REAL as the reference
                            (src/rungeKutta.cu:326-333); 1: |sum (c_i - c*_i) k_i|
                            (no cancellation against x), with t and dt kept in
                            double by the controller                           */
    double  p0Amp;       /* pressure profile p0(X) = beta*(1 + p0Amp*exp(-r^2/p0Width^2));
                            p0Amp = 0 gives the reference's uniform p0 = beta  */
    double  p0Width;
    int32_t stageKernel; /* 0: TMA-fed stage kernel (default); 1: the generic
                            tiled stage kernel (plain loads), kept for
                            cross-checks of the former  */
    int32_t reserved[7];
} gm_params;

/* Result of one attempted adaptive step (src/main.cu:259-384). */
typedef struct gm_step_result {
    double  maxDelta;    /* max over points and components of the error norm  */
    double  t;           /* time after the step                                */
    double  dt;          /* step size for the next attempt                     */
    int32_t accepted;    /* 1 if maxDelta < maxError                            */
    int32_t timeIndex;   /* accepted-step counter after the step                */
    uint32_t status;     /* GM_ST_* bits                                        */
    int32_t pad;
} gm_step_result;

/* Device-resident controller state. */
typedef struct gm_state {
    double  t, dt, maxDelta;
    int32_t timeIndex;   /* accepted steps so far (main.cu loop index)          */
    int32_t nAttempted;  /* attempted steps so far                              */
    int32_t nRejected;
    uint32_t status;
    double  dtUsed;      /* step size of the last attempted step (the dt that
                            writeTs prints, main.cu:357)                        */
    int32_t event;       /* GM_EV_* bits of the step gm_run_events stopped at   */
    int32_t pad;
} gm_state;

/*
 * Reductions (src/diagnostics.cu:12-134 and src/maths.cu) plus the force-free
 * residual this library adds.  All accumulate in double.
 */
typedef struct gm_reduction {
    double B2;           /* sum B^2 detJac with 1/2,1/4,1/8 boundary weights * dx dy dz (maths.cu:647-680) */
    double BMax;         /* max |B| over inner points                           */
    double JMax;         /* max |J| (diagnostics.cu:15-22)                      */
    double JxB_B2Max;    /* max |JxB|/B^2 (maths.cu:168-200)                    */
    double residual;     /* force-free residual sum|JxB| / sum(|J||B|) over inner points: the
                            |J||B|-weighted mean of sin(angle(J,B))                          */
    double residualPw;   /* unweighted mean over inner points of |JxB|/(|J||B|); points with
                            |J||B| = 0 count as 0                                            */
    double minDetJac;    /* min detJac over inner points and the ghost planes of
                            non-periodic faces                                  */
    double wedgeMin;     /* min of the 8 corner wedge products (maths.cu:497-569) */
    double convex;       /* 1 if every inner point is convex, -1 otherwise (maths.cu:573-643) */
    double errB_1ez;     /* rms |B - e_z| (maths.cu:294-328)                    */
    double errXb_XbAn;   /* rms |x - x_analytic| (maths.cu:332-377)             */
    double epsilonStar;  /* force-free parameter eps* along the central column
                            (maths.cu:203-290, diagnostics.cu:32-47)            */
    double U2;           /* inertia: sum |u|^2 detJac with the boundary weights of B2
                            * dx dy dz (maths.cu:684-710, diagnostics.cu:114-122); 0 without */
    double UMax;         /* inertia: max |u| (diagnostics.cu:124-130); 0 without        */
} gm_reduction;

typedef struct gm_handle gm_handle;

/* ---- parameters ---------------------------------------------------------- */

/* Fill p with the namelist defaults of src/readNamelist.f90:92-150 at the given
 * precision (32 or 64), including the single-precision literal rounding of
 * those defaults, and derive dx..dz1 (readNamelist.f90:185-186). */
int gm_params_default(gm_params* p, int precision);

/* Recompute dx = Lx/(nx-1), dx1 = 1/dx, ... in the run precision
 * (src/readNamelist.f90:185-186). */
int gm_params_derive(gm_params* p);

/* Read ./params.in style namelists (&comp &start &run &io) from `path` on top
 * of gm_params_default (src/readNamelist.f90:152-178). */
int gm_params_read(gm_params* p, const char* path, int precision);

/* ---- initial state (src/init.cu:30-384, 388-419; boundaries.cu:492-634) -- */

/* Build the initial B0 and grid xb on the host, ghost layers included, as
 * initState + initDistortion + setPeriHost + setGridPeriHost do.  Supports
 * bInit "blobs", "homZ", "analytic" and initDist "none", "initShearX",
 * "centerShift".  (gm_create still refuses initShearA/B != 0: the
 * ghost-plane correction of distorted grids, addDist, is not in the stage
 * kernels.) */
int gm_init_state(const gm_params* p, void* B0, void* xb);

/* ---- handle lifecycle (src/memory.cu:10-95, main.cu:181-256) ------------- */

/* Allocate a relaxation for the parameters p (as read from params.in).
 * Accepted: jMethod "Stokes" (the TMA stage kernel), "Stokes4th",
 * "StokesQuint", "StokesTri" and "Classic" (current.cu:10-1681, selected as
 * in current.cu:1685-1712); inertia, jxbAver and the Classic pressure
 * gradient.  Anything else (another jMethod or pMethod, initShearA/B != 0)
 * returns GM_EPARAM with the reason in gm_last_error(). */
int gm_create(const gm_params* p, gm_handle** out);
int gm_destroy(gm_handle* h);
/* Use `stream` (a cudaStream_t) for all work of h; NULL selects the handle's
 * own non-blocking stream. */
int gm_set_stream(gm_handle* h, void* stream);

/* Copy the initial state to the device (src/main.cu:181-232).  xb and B0
 * (reference layout) may be host or device arrays. */
int gm_upload(gm_handle* h, const void* xb, const void* B0, double t, double dt);

/* ---- the relaxation hot path -------------------------------------------- */

/* One Runge-Kutta stage n (0..5) at the current dt: B = jac.B0/Delta
 * (rungeKutta.cu:28-108) with ghost fill (boundaries.cu:637-658), the Stokes
 * current (current.cu:222-409) and k_n = dt eps JxB plus the incremental stage
 * position (rungeKutta.cu:112-247).  Stage 5 also forms x_new, x* and the
 * error norm (rungeKutta.cu:251-353).  Exposed for stage-level parity tests. */
int gm_stage(gm_handle* h, int n);

/* Accept/reject and dt update from the error norm of the last stage 5
 * (src/main.cu:317-383), done on the device. */
int gm_control(gm_handle* h);

/* One attempted adaptive step (6 stages + control), synchronous; fills r. */
int gm_step(gm_handle* h, gm_step_result* r);

/* Enqueue `nSteps` attempted steps without synchronising (CUDA-graph replay).
 * Steps after the stop rule (timeIndex >= nCycle or dt <= dtMin) do no work. */
int gm_steps_async(gm_handle* h, int nSteps);

/* Run until nCycle accepted steps (counted from the handle's timeIndex) or
 * dt <= dtMin, as the loop of src/main.cu:259-384 (without its file output). */
int gm_run(gm_handle* h, int nCycle, gm_state* out);

/* As gm_run, but also stop after every accepted step whose output is due
 * (the nTs, dtDump, dtSave and last-step triggers of src/main.cu:355-377,
 * from the handle's parameters); out->event then holds the GM_EV_* bits,
 * out->dtUsed the step size of that step and out->dt the adapted one.  Call
 * again to continue; nCycle counts from the handle's timeIndex of the first
 * call after gm_upload or gm_set_dt. */
int gm_run_events(gm_handle* h, int nCycle, gm_state* out);

/* Read the device controller state (synchronises the handle's stream). */
int gm_get_state(gm_handle* h, gm_state* out);
int gm_set_dt(gm_handle* h, double t, double dt, int timeIndex);

/* Recompute B, detJac (ghosts included) and J at the current grid, as the
 * post-accept refresh does (src/main.cu:342-353), and evaluate the reductions
 * (src/diagnostics.cu:12-134).  r may be NULL. */
int gm_refresh(gm_handle* h, gm_reduction* r);

/* Copy state to host arrays (any may be NULL): xb, B ghosted AoS; J inner AoS;
 * detJac ghosted scalar -- the arrays prepareDump copies
 * (src/diagnostics.cu:138-152).  B, J and detJac are those of the last
 * gm_refresh. */
int gm_download(gm_handle* h, void* xb, void* B, void* J, void* detJac);

/* Grid-quality fields at the current grid, inner layout i + nx*(j + ny*k)
 * (any may be NULL): the signed cell volume (dirCellVol, maths.cu:441-490),
 * the convexity flag +-1 (gridConvexity, maths.cu:573-643) and the minimum of
 * the 8 corner wedge products (gridWedgeMin, maths.cu:494-569). */
int gm_grid_fields(gm_handle* h, void* cellVol, void* convexity, void* wedgeMin);

/* Autotuner of the stage kernel's z-chunk depth (the planes one CTA
 * marches through): times `trials` rounds of stages 0..4 on the uploaded
 * state for each candidate depth (the cost model's best eight and the current
 * one) with CUDA events on the handle's stream, keeps the fastest and
 * recaptures the step graph.  Stages 0..4 write only the stage buffers, so
 * the state a run starts from is unchanged; results do not depend on the
 * depth.  Call after gm_upload; *tz and *ms (mean time of stages 0..4) may be
 * NULL.  No counterpart in the reference (its block shape is fixed,
 * src/main.cu:130-137). */
int gm_autotune(gm_handle* h, int trials, int* tz, double* ms);
/* Set the stage kernel's z-chunk depth directly (1..nz; the TMA stage kernel
 * only), e.g. to repeat a depth gm_autotune chose; the step graph is
 * recaptured.  No counterpart in the reference. */
int gm_set_tile_z(gm_handle* h, int tz);
/* Failure-detection test hook (no counterpart in the reference, which has no
 * bounded waits).  While `on` is non-zero, the TMA stage kernel's copy
 * producer withholds the copies of each tile's first position planes, so
 * every CTA's bounded wait for them (2^22 polls each) runs out: the CTA
 * records GM_ST_TIMEOUT in the status word, waits (bounded) for the copies
 * it did issue and returns; the step is neither accepted nor used to adapt
 * dt, and the run stops with GM_ETIMEOUT.  No copy is left in flight and no
 * wait is unbounded; the device context stays usable.  The step graph is
 * recaptured.  GM_EPARAM when the run does not use the TMA stage kernel.
 * Off by default. */
int gm_debug_stall(gm_handle* h, int on);

/* Stage increments k_0..k_4 of the last step (inner AoS in the reference kk
 * layout src/rungeKutta.cu:236: 3*nx*ny*nz values each, or 6*nx*ny*nz with
 * inertia, the position increment then the velocity increment per point)
 * -- for stage parity tests. */
int gm_download_k(gm_handle* h, int m, void* k);

/* Grid buffers of the last step in the reference layout (ghosted AoS):
 * which = 0..4: stage position x_{which+1} written by stage `which`
 * (the xb_tmp of src/rungeKutta.cu:234); 5: x_6, the start grid of a
 * rejected retry; 6: x_new of the combine (src/rungeKutta.cu:345). */
int gm_download_x(gm_handle* h, int which, void* xb);

/* Velocity of an inertia run (inertia = T), inner points, AoS 3*nx*ny*nz in
 * the layout of the reference's uu (src/global.h:143, rungeKutta.cu:147-150).
 * gm_upload zeroes it (uInit = "nil", src/init.cu:362-364); gm_upload_u, after
 * gm_upload, sets the velocity of the step start (the restart path,
 * src/io.cu:466-481).  gm_download_u: which = 0..4: stage velocity u_{which+1}
 * (uu_tmp of src/rungeKutta.cu:238-241); 5: the current velocity (u_6, the
 * start of a rejected retry, or the accepted u_new); 6: u_new of the last
 * combine (uu_new, src/rungeKutta.cu:345-350).  GM_EPARAM without inertia. */
int gm_upload_u(gm_handle* h, const void* u);
int gm_download_u(gm_handle* h, int which, void* u);

/* Largest nz that gm_reduce_noalloc accepts: the number of per-plane partial
 * sums its fixed scratch array holds. */
#define GM_NOALLOC_MAX_PLANES 4096

/* The reductions of gm_refresh computed from fields the caller already holds
 * on the device, without allocating any device memory.  This entry point has
 * no counterpart in the reference.  It is for callers that cannot allocate at
 * the point where they want diagnostics: applications whose device memory
 * belongs to their own pool allocator (a cudaMalloc from a library fails or
 * escapes the pool's accounting), stream-ordered pipelines that must not
 * stall (cudaFree, and cudaMalloc in places, synchronise the device), and
 * services that allocate nothing after start-up.
 *   B, J, detJac: DEVICE arrays of REAL in the layouts gm_download returns
 *                 (B ghosted AoS, J inner AoS, detJac ghosted scalar).
 *   out:          DEVICE pointer to one gm_reduction; wedgeMin, convex and
 *                 errXb_XbAn need the grid and U2, UMax the velocity: they
 *                 are set to NaN; epsilonStar is not written.
 *   stream:       cudaStream_t to run on (NULL: the legacy default stream).
 * The per-plane partial sums live in one fixed device array of
 * GM_NOALLOC_MAX_PLANES x 16 doubles (512 KiB, held by every GPU that loads
 * the library until the process exits); nz above GM_NOALLOC_MAX_PLANES is
 * rejected with GM_EPARAM.  Each call overwrites every partial it reads, so
 * nothing has to be cleared between calls, but all calls share that array:
 * calls that overlap on the GPU (concurrent streams) race.  The first call on
 * a device looks up the array's device address with that device current (a
 * failed lookup is retried by the next call); make that first call before any
 * stream capture.  A CUDA error left pending by the caller is reported
 * (GM_ECUDA) and left pending, and nothing is launched.  No cudaMalloc,
 * cudaFree or allocating library routine is called. */
int gm_reduce_noalloc(const gm_params* p, const void* B, const void* J, const void* detJac,
                      gm_reduction* out, void* stream);

/* ---- many independent cases (no counterpart in the reference, which runs
 * one case per process) ------------------------------------------------------
 * Cases of uneven grid sizes advance together: each Runge-Kutta stage is ONE
 * persistent launch whose CTAs take 32 x 8 x 32 tiles of every case from a
 * work counter, one launch runs every case's controller (src/main.cu:321-383
 * per case), and a step of all cases is one CUDA graph replay.  A case whose
 * controller has stopped (nCycle, dtMin, NaN) or that gm_batch_stop /
 * gm_batch_run stopped is skipped by the launches.  All cases share the
 * precision and the pressure flag; each has its own dt and time. */
typedef struct gm_batch gm_batch;

/* Outcome of one case of gm_batch_run. */
typedef struct gm_batch_case {
    double  seconds;     /* wall time from the start of gm_batch_run to the check that ended the case */
    double  residual;    /* residual at that check (weighted, or pointwise when asked) */
    double  t, dt;
    int32_t attempted, accepted;
    uint32_t status;     /* GM_ST_* bits */
    int32_t converged;   /* 1 when the residual reached the target */
} gm_batch_case;

int gm_batch_create(const gm_params* cases, int nCases, gm_batch** out);
int gm_batch_destroy(gm_batch* b);
/* Autotuner of the batched work-item depth (planes per tile: 16, 32 or 64),
 * timed as gm_autotune does over the batched stages 0..4; call after every
 * case is uploaded.  No counterpart in the reference. */
int gm_batch_autotune(gm_batch* b, int trials, int* tzb, double* ms);
int gm_batch_upload(gm_batch* b, int c, const void* xb, const void* B0, double t, double dt);
/* Enqueue nSteps attempted steps of every case (graph replays, no sync). */
int gm_batch_steps_async(gm_batch* b, int nSteps);
int gm_batch_get_state(gm_batch* b, int c, gm_state* out);
int gm_batch_refresh(gm_batch* b, int c, gm_reduction* r);
int gm_batch_download(gm_batch* b, int c, void* xb, void* B, void* J, void* detJac);
/* Stop case c: the launches skip it from the next step on. */
int gm_batch_stop(gm_batch* b, int c);
/* Advance all cases; every checkEvery steps each running case's residual
 * (gm_reduction.residual, or residualPw when pointwise != 0) is evaluated and
 * a case at or below `residual` is stopped.  Cases also stop at nCycle
 * accepted steps (counted from this call) or by their own stop rule.  Returns
 * when every case has stopped; out[c] (may be NULL) gets each case's outcome. */
int gm_batch_run(gm_batch* b, int nCycle, double residual, int pointwise, int checkEvery, gm_batch_case* out);
int64_t gm_batch_launch_count(const gm_batch* b);

/* ---- learned warm start (no counterpart in the reference) ---------------- */

/* Check of the tensor-core MMA core: D[128 x N] = A[128 x K] . B[N x K]^T
 * with BF16 operands (DEVICE arrays, row-major) and FP32 accumulation in
 * tensor memory; N, K multiples of 16 in [16, 256].  *status (device int) is
 * set to 1 if the completion wait gave up.  Synchronises the device. */
int gm_nn_tc_gemm_check(const void* A, const void* B, float* D, int N, int K, int* status);

/* The network's layers (glemur_gb300/warmstart.py drives them).  Activations
 * are DEVICE arrays of BF16, channels-last (voxel v = x + nx (y + ny z)),
 * passed as views: a pointer (16-byte aligned) and a channel stride ld (a
 * multiple of 8).  Grids are periodic in x / y when xper / yper, zero-padded
 * in z.  All calls enqueue on `stream` (a cudaStream_t) and do not
 * synchronise; a tensor-core completion wait that gives up sets *status.
 *
 * gm_nn_conv: 3x3x3 convolution as an implicit GEMM on the tensor cores.
 *   out[v][o] = sum_t sum_i in[v + off(t)][i] W[t][o][i] (+ bias[o]), ReLU if
 *   relu, then times (mask[v][o] > 0) if mask; the input is the concatenation
 *   of the views in1 (c1 channels, c1 a multiple of 8) and in2 (c2); W is
 *   BF16 [27][Np][Kc] (Kc >= c1 + c2 and Np >= co multiples of 16, <= 256).
 *   With W flipped in t and transposed it is the input gradient.  A CTA takes
 *   128 voxels and all Np outputs, or a slice of them when the two operand
 *   stages would not fit its shared memory. */
int gm_nn_conv(const void* in1, int ld1, int c1, const void* in2, int ld2, int c2, const void* W, const float* bias,
               void* out, int ldo, int co, const void* mask, int ldm, int relu, int nx, int ny, int nz, int xper,
               int yper, int Kc, int Np, int* status, void* stream);
/* dW[t][o][i] += sum_v dout[v][o] in[v + off(t)][i] (FP32, i < ci <= c1 +
 * c2, o < co <= 256), on the tensor cores: one GEMM per chunk of vchunk voxels
 * (a multiple of 64; 0 lets the library choose) with the 27 taps' input
 * channels stacked as its rows, in tiles of 128.  dout is read up to co
 * rounded up to 8 channels, the input views up to ci rounded up to 8; every
 * view starts on 16 bytes with a channel stride that is a multiple of 8. */
int gm_nn_conv_wgrad(const void* dout, int ldd, int co, const void* in1, int ld1, int c1, const void* in2, int ld2,
                     int c2, float* dW, int ci, int nx, int ny, int nz, int xper, int yper, int vchunk, int* status,
                     void* stream);
/* db[o] += sum_v d[v][o]. */
int gm_nn_bias_grad(const void* d, int ld, int c, long long V, float* db, void* stream);
/* 2x2x2 mean pooling of the fine grid (nx, ny, nz) and its adjoint
 * (backward: the fine gradient from the coarse one, added when accumulate). */
int gm_nn_pool(const void* in, int ldi, void* out, int ldo, int c, int nx, int ny, int nz, int backward,
               int accumulate, void* stream);
/* Nearest 2x upsampling to the fine grid (nx, ny, nz) and its adjoint. */
int gm_nn_upsample(const void* in, int ldi, void* out, int ldo, int c, int nx, int ny, int nz, int backward,
                   void* stream);
/* d *= (y > 0). */
int gm_nn_relu_bwd(void* d, int ldd, const void* y, int ldy, int c, long long V, void* stream);
/* loss += scale sum (y - tgt)^2 over channels 0..2 and planes 1..nz-2;
 * dy = 2 scale (y - tgt) there and 0 on the first and last planes; tgt FP32
 * [V][3], moved by the translation (sx, sy) and symmetry `sym` as
 * gm_nn_input's input. */
int gm_nn_mse(const void* y, int ldy, const float* tgt, void* dy, int lddy, int nx, int ny, int nz, float scale,
              float* loss, int sx, int sy, int sym, void* stream);
/* Adam step t (t = 0: no update) of FP32 W[27][co][ci], b[co] with their
 * moments and gradients, then the BF16 operand layouts Wf[27][Npo][Kci]
 * (forward) and Wb[27][Npi][Kco] (input gradient: taps flipped, transposed)
 * and the padded bias. */
int gm_nn_adam(float* W, float* mW, float* vW, const float* gW, float* b, float* mb, float* vb, const float* gb, int co,
               int ci, float lr, float b1, float b2, int t, float eps, void* Wf, int Npo, int Kci, void* Wb, int Npi,
               int Kco, float* bpad, void* stream);
/* Network input from B0 on the device (reference layout, REAL of
 * `precision`): channels (B0x, B0y, B0z - 1) of the inner points, ld
 * channels, the sample moved by a symmetry of the periodic cross-section for
 * data augmentation: cell (i, j) reads the source cell u = (i + sx) mod nx,
 * v = (j + sy) mod ny (0 <= sx < nx, 0 <= sy < ny), then, by the bits of
 * `sym` (0..7), 4: u <-> v (nx == ny only), 2: v -> ny - 1 - v, 1: u -> nx -
 * 1 - u; the vector's x, y components follow as polar vectors (x negated for
 * bit 1, y for bit 2, then swapped for bit 4). */
int gm_nn_input(const void* B0, int precision, int nx, int ny, int nz, void* x, int ld, int sx, int sy, int sym,
                void* stream);
/* Test-time translation averaging of the warm-start network: the displacement
 * channels 0..2 of an output y (BF16 [V][ldy], in grid spacings) computed on
 * the input translated by (sx, sy) (gm_nn_input), moved back to the grid's
 * own cells, times w, written to d (float [V][3], device) when `first`, else
 * added.  No counterpart in the reference. */
int gm_nn_disp_accumulate(const void* y, int ldy, int nx, int ny, int nz, int sx, int sy, float w, int first,
                          float* d, void* stream);
/* Warm-start grid on the device: the displacement d (float [V][3], grid
 * spacings) smoothed by `passes` 3x3x3 box filters (periodic x / y as p
 * selects, zero beyond z), added to the identity grid xid (device, reference
 * layout, REAL of p->precision) at the inner points except the first and last
 * z-planes, with periodic x / y ghosts as images of the opposite inner points
 * shifted by -/+ (L + d); written to xb (device, same layout).  scratch:
 * device floats, 6 nx ny nz.  No counterpart in the reference (its runs start
 * from the identity grid). */
int gm_nn_warm_grid(const float* d, const gm_params* p, int passes, const void* xid, float* scratch, void* xb,
                    void* stream);
/* Zero `bytes` bytes of device memory (cudaMemsetAsync). */
int gm_nn_zero(void* p, size_t bytes, void* stream);
/* Failure-detection test hook for the tensor-core convolutions (no
 * counterpart in the reference): while `on` is non-zero (process-wide, read
 * at each launch of gm_nn_conv / gm_nn_conv_wgrad), every CTA first waits on
 * an mbarrier that nothing arrives on, with a limit of 2^10 polls; the wait
 * runs out before any MMA is issued, the CTA frees its tensor memory and sets
 * *status = 1, and its output is left unwritten.  Off by default. */
int gm_nn_debug_stall(int on);

/* Number of CUDA devices and selection of the device the calling thread
 * uses (the cudaGetDeviceCount / cudaSetDevice of src/main.cu:47-80). */
int gm_device_count(int* n);
int gm_set_device(int dev);

/* ---- run-directory files (src/io.cu), host only ------------------------- */
/* Arrays are REAL of p->precision in the reference layouts above; files are
 * legacy VTK with big-endian binary payloads, byte for byte as io.cu writes
 * them.  All return GM_OK or GM_EIO. */

/* cuda.info (io.cu:10-82) for the devices of this machine. */
int gm_io_write_cuda_info(const char* path, int precision, long activeDevice);
/* data/B0.vtk: STRUCTURED_POINTS, ghosts included (io.cu:167-205). */
int gm_io_write_b0(const gm_params* p, const char* path, const void* B0);
/* data/dump<n>.vtk or data/save.vtk: STRUCTURED_GRID with the 9 parameter
 * fields, POINTS xb, VECTORS bfield, with inertia VECTORS ufield (zero
 * ghosts) and, as p->dump* select, VECTORS jfield (zero ghosts), SCALARS
 * detJac / cellVol / convexity / wedgeMin (io.cu:209-386, 503-538).  J, u,
 * cellVol, convexity, wedgeMin are inner layout; the others ghosted.  u may be
 * NULL when p->inertia is 0. */
int gm_io_write_dump(const gm_params* p, const char* path, double t, double dt, const void* xb, const void* B,
                     const void* J, const void* detJac, const void* cellVol, const void* convexity,
                     const void* wedgeMin, const void* u);
/* Restart: t, dt and xb (and, with inertia, the velocity u, inner AoS) from a
 * save file, B0 from a B0 file (io.cu:390-499).  Grid sizes come from p, as in
 * the reference, which passes its parameters to readState by value.  The
 * reference skips the B block before the velocity with a read that starts at
 * the "VECTORS bfield" line (io.cu:468-473) and finds the velocity only when
 * the end of the B block holds no newline byte; here the file is read block
 * by block. */
int gm_io_read_state(const gm_params* p, const char* save_path, const char* b0_path, void* xb, void* B0,
                     double* t, double* dt, void* u);
/* One time-series line (io.cu:542-678) into buf: the header line when
 * header != 0 (toFile != 0 labels the error column "maxDelta" as the file
 * does, else "maxError" as stdout does), else the row for (it, t, dt,
 * maxDelta) with the reductions p->red* select; B2f = B2 - B2res.  Returns
 * the length written, or GM_EPARAM when buf is too small. */
int gm_io_ts_line(const gm_params* p, const gm_reduction* r, double B2res, double t, double dt, int it,
                  double maxDelta, int header, int toFile, char* buf, int bufSize);

/* Cumulative kernel launches issued by this handle (for accounting). */
int64_t gm_launch_count(const gm_handle* h);

const char* gm_last_error(void);
const char* gm_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GLEMUR_H_ */
