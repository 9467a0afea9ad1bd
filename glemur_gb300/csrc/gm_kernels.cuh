// gm_kernels.cuh -- device kernels of the relaxation hot path.
//
// One Runge-Kutta stage is one kernel launch.  Each CTA owns a column tile of
// TX x TY points and marches through a chunk of TZ planes.  Grid positions of
// the stage are read plane by plane into a ring of 5 shared-memory planes
// (tile + 2-point halo); B = jac.B0/Delta is computed once per point on the
// tile + 1-point face halo into a ring of 4 B planes; the Stokes current J,
// the stage increment k_n = dt eps (J x B) [- dt grad p] and the next stage
// position are formed at the tile points.  Stage 5 also forms x_new, x* and
// the error norm and reduces its maximum.  So the reference's per-stage
// sequence B_JacB0 + updateBbound + setPeriFace + JStokes + kk + setGridPeri
// + cudaMemcpy (src/main.cu:260-307) and xNewStar + findDevMax
// (main.cu:309-319) become six launches per step, and the accept/reject rule
// (main.cu:321-383) a seventh single-thread launch.
//
// Storage (all SoA, component-major):
//   positions: padded with 2 ghost layers per side, index
//              (i+2) + px*((j+2) + py*(k+2)), component stride cs.  Periodic
//              ghost layers hold the shifted images x -/+ (L + d) of the inner
//              points (boundaries.cu:532-582), written by the stage that
//              produces the positions; non-periodic ghost layers hold the
//              fixed line-tied positions of the initial grid.
//   B0:        same padded layout (ghost depth 1 used).
//   k_m:       inner points only, index i + kpx*(j + ny*k) with the row pitch
//              kpx = nx rounded up to 8 (so rows start on 16-byte boundaries,
//              as tensor-map copies need), component stride kcs.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gmk {

constexpr int TX = 32;          // tile width in x = one warp
constexpr int XRING = 5;        // planes of positions held in shared memory
constexpr int BRING = 4;        // planes of B held in shared memory

// Device-resident controller state (one per handle).
struct DevState {
    double t, dt, maxDelta;
    unsigned long long maxDeltaBits;   // running max of the error norm (bits of a non-negative double)
    int timeIndex;                     // accepted steps (main.cu loop index)
    int nAttempted, nRejected;
    int cur;                           // which of X[0], X[1] holds the step's start grid
    int target;                        // stop once timeIndex >= target
    unsigned status;                   // GM_ST_* bits
    int done;
    int logCap;
    int lastAccepted;                  // outcome of the last attempted step
    double dtUsed;                     // step size of the last attempted step
    int event;                         // GM_EV_* bits of the last accepted step
    int eventsOn;                      // stop (done) after an accepted step with output due
};

// Kernel-side run parameters (passed by value; REAL = T).
template <typename T>
struct KP {
    int nx, ny, nz;
    int px, py, pz;          // padded extents
    long long cs;            // component stride of padded arrays
    long long N;             // nx*ny*nz
    int kpx;                 // row pitch of the k_m arrays (nx rounded up to 8)
    long long kcs;           // component stride of the k_m arrays
    T dx, dy, dz, dx1, dy1, dz1;
    T hdx1, hdy1, hdz1;      // dx1/2, dy1/2, dz1/2 (exact)
    T Lx, Ly, Lz, Ox, Oy, Oz;
    int xPeri, yPeri, zPeri, zUpdate, errMode, refDt;
    int jClassic;            // jMethod = "Classic": the finite-difference current (generic kernel only)
    int jOct;                // jMethod = "Stokes4th": J from the octilateral pass (outJ; generic kernel only)
    int jQuint;              // jMethod = "StokesQuint": J from the quintilateral pass (outJ; generic kernel only)
    int jTri;                // jMethod = "StokesTri": J from the same pass in its triangle-only form
    int inertia;             // the velocity equation (generic kernel only)
    T nu;                    // velocity damping
    int jxbAver;             // neighbour-averaged Lorentz force (generic kernel only)
    T jxbW;                  // its weight
    T beta, p0Amp, p0W2;     // pressure: p0(X) = beta (1 + p0Amp exp(-(X^2+Y^2)/p0W2))
    T inv_p0W2;              // 1 / p0W2
    double maxError, dtMin;  // run-precision values widened to double
    T db[6][6];              // b[n+1][m] - b[n][m] of the Cash-Karp tableau
    T c[6], cst[6];          // 5th- and 4th-order weights
    double cmc[6];           // c - c* in double (error norm of errMode 1)
    T cmcT[6];               // c - c* in the run precision
    T inv8dxdydz;            // 1 / (8 dx dy dz): det(a, b, c) -> Delta
    double ar, az, phi1;     // analytic-field parameters (distance-to-analytic diagnostic)
    int shear;               // initShearA or initShearB != 0: addDist on the line-tied z ghost planes
    int initDistCode;        // 0: initShearX, 1: centerShift (src/readNamelist.f90)
    T shA, shB, shK;         // initShearA, initShearB, initShearK
    const T* shearTab;       // with shear: the z ghost planes' corrected positions (k_shear_table)
    int wantXbAn;
    int nTs;                 // output cadences (main.cu:355-377)
    T dtDump, dtSave;
    const T* ex;             // epsilon profile factors per axis (rungeKutta.cu:180-185)
    const T* ey;
    const T* ez;
};

enum { MODE_STAGE = 0, MODE_DIAG = 1 };

// Reduction partial of one CTA (diagnostic mode).
enum {
    R_SUM_CROSS = 0, R_SUM_JB, R_SUM_PW, R_SUM_B2W, R_SUM_E1, R_SUM_E2, R_SUM_U2,
    R_MAX_JXBB2, R_MAX_B, R_MAX_J, R_MAX_U,
    R_MIN_DET, R_MIN_WEDGE, R_MIN_CONVEX,
    R_COUNT
};
constexpr int R_LAST_SUM = R_SUM_U2, R_LAST_MAX = R_MAX_U;   // sums, then maxima, then minima

template <typename T>
struct StageArgs {
    KP<T> p;
    T* X[2];                 // start / new grid (roles swap on accept)
    T* XS[2];                // stage positions, ping-pong
    T* K[5];                 // k_0..k_4
    T* U[2];                 // inertia: velocity at the step start / of the new step (roles follow X)
    T* US[2];                // inertia: stage velocities, ping-pong
    T* KU[5];                // inertia: velocity increments k_u,0..k_u,4
    const T* B0;
    const T* B0s;            // B0 scaled by (4 dy dz, 4 dx dz, 4 dx dy), padded layout
    DevState* st;
    double* log;             // per attempt: maxDelta, dt after the update, accepted
    int n;                   // stage index 0..5
    int TZ;                  // planes per CTA
    int jpass;               // diagnostic mode on the stage's own input grid (the J pass of jxbAver)
    int stall;               // failure-detection test (gm_debug_stall): the TMA stage kernel withholds the
                             // copies of each tile's first position planes
    // diagnostic mode outputs (reference layout) and partials
    T* outB;                 // ghosted AoS
    T* outJ;                 // inner AoS
    T* outD;                 // ghosted scalar detJac
    double* part;            // R_COUNT per CTA
};

// Host-side launchers (explicitly instantiated for float and double).
template <typename T>
cudaError_t launch_j_oct(const StageArgs<T>& a, cudaStream_t s);
template <typename T>
cudaError_t launch_j_quint(const StageArgs<T>& a, cudaStream_t s);
template <typename T>
cudaError_t launch_stage(const StageArgs<T>& a, int mode, int pressure, dim3 grid, dim3 block, size_t smem,
                         cudaStream_t s);
template <typename T>
size_t stage_smem_bytes(int TY, int mode, int pressure);
template <typename T>
cudaError_t prepare_kernels();
template <typename T>
int stage_occupancy(int TY, int pressure, size_t smem);
template <typename T>
cudaError_t launch_control(const KP<T>& p, DevState* st, double* log, cudaStream_t s);
template <typename T>
cudaError_t launch_finalize(const double* part, int nparts, double* out, cudaStream_t s);
// ghosted AoS (reference layout) <-> padded SoA
template <typename T>
cudaError_t launch_unpack(const KP<T>& p, const T* aos, T* soa, cudaStream_t s);
template <typename T>
cudaError_t launch_pack(const KP<T>& p, const T* soa, T* aos, cudaStream_t s);
template <typename T>
cudaError_t launch_images(const KP<T>& p, T* soa, cudaStream_t s);
template <typename T>
cudaError_t launch_scale_b0(const KP<T>& p, const T* B0, T* B0s, cudaStream_t s);
template <typename T>
cudaError_t launch_shear_table(const KP<T>& p, const T* X, T* tab, cudaStream_t s);
template <typename T>
cudaError_t launch_pack_k(const KP<T>& p, const T* k, T* aos, cudaStream_t s);
template <typename T>
cudaError_t launch_pack_k6(const KP<T>& p, const T* kx, const T* ku, T* aos, cudaStream_t s);
template <typename T>
cudaError_t launch_unpack_k(const KP<T>& p, const T* aos, T* k, cudaStream_t s);
template <typename T>
cudaError_t launch_export_ghosts(const KP<T>& p, T* outB, T* outD, cudaStream_t s);
// grid-quality fields (inner layout) of a padded grid
template <typename T>
cudaError_t launch_grid_fields(const KP<T>& p, const T* X, T* cellVol, T* convexity, T* wedgeMin, cudaStream_t s);
// eps* of the central column from the exported B (ghosted AoS), J (inner AoS)
// and the padded grid, into *out; scratch holds 2 nz REALs
template <typename T>
cudaError_t launch_eps_star(const KP<T>& p, const T* B, const T* J, const T* X, T* scratch, double* out,
                            cudaStream_t s);

// TMA-fed stage kernel (gm_stage_tma.cuh): 32 x 8 tiles, operand planes
// streamed by cp.async.bulk.tensor.  tm[0..3] are the tensor maps of X[0],
// X[1], XS[0], XS[1] and tm[4] of B0s (box 36 x 12 x 1 x 3 over (px, py, pz,
// component)); tm[5..9] those of k_0..k_4 (box 32 x 8 x 1 x 3 over
// (nx, ny, nz, component) with row pitch kpx).
template <typename T>
struct StageArgsTMA {
    CUtensorMap tm[10];
    StageArgs<T> a;
};
template <typename T>
size_t stage_tma_smem_bytes(int pressure, int n);
template <typename T>
cudaError_t prepare_stage_tma();
template <typename T>
int stage_tma_occupancy(int pressure);
template <typename T>
cudaError_t launch_stage_tma(const StageArgsTMA<T>& A, int pressure, dim3 grid, cudaStream_t s);
// Row groups of the single-case FP32 pressure stage kernel's tile (32 x 8
// STAGE_ROWS columns) and the tile heights of the single-case and batched
// launches.
#ifndef GM_STAGE_ROWS
#define GM_STAGE_ROWS 2
#endif
constexpr int STAGE_ROWS = GM_STAGE_ROWS;
constexpr int STAGE_BATCH_TY = 8;
// Two row groups pay where a point has much work (the pressure gradient:
// 30.6 against 28.9 G cell-RK-stages/s on 256x256x512); without it the third
// CTA per SM that one row group allows is worth more (36.3 against 34.7 G on
// the 128x128x256 braid).  FP64 keeps one: two would not fit two CTAs'
// shared memory per SM.
template <typename T, bool PRESS>
constexpr int stage_rows() { return (sizeof(T) == 4 && PRESS) ? STAGE_ROWS : 1; }
template <typename T>
inline int stage_tma_ty(int pressure) { return 8 * (pressure ? stage_rows<T, true>() : stage_rows<T, false>()); }
// Batched stage launch: `work` holds (case, bx, by, bz) items over the
// device array `cases`; `counter` is this stage's work counter (zero on
// entry).  `nblocks` CTAs, persistent.
template <typename T>
cudaError_t launch_stage_tma_batch(const StageArgsTMA<T>* cases, const int4* work, int nwork, int* counter, int n,
                                   int pressure, int nblocks, cudaStream_t s);
template <typename T>
int stage_tma_batch_occupancy(int pressure);
// The controllers of all cases of a batch (and the re-arm of the counters).
template <typename T>
cudaError_t launch_control_batch(const StageArgsTMA<T>* cases, int ncases, int* counters, cudaStream_t s);

}  // namespace gmk
