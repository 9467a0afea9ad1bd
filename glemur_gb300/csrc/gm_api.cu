// gm_api.cu -- the C-ABI of include/glemur.h over the relaxation kernels.
//
// A handle owns every device buffer of one relaxation (src/memory.cu:10-95
// allocates the reference's), a stream, the device-resident controller state
// and a CUDA graph of one attempted step (6 stage launches + the control
// launch), so a run is graph replays with no host round trip per step; the
// reference instead synchronises after every launch and copies maxDelta to the
// host each step (src/main.cu:259-384, src/maths.cu:101-130).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "glemur.h"
#include "gm_internal.h"
#include "gm_kernels.cuh"

using gmk::DevState;
using gmk::KP;
using gmk::StageArgs;
using gmk::StageArgsTMA;

namespace {

#define CUDA_TRY(x)                                                                        \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess)                                                             \
            return gm::fail(GM_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_));    \
    } while (0)

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    }
    return fn;
}

int check_params(const gm_params* p) {
    if (!p) return gm::fail(GM_EPARAM, "null params");
    if (p->precision != 32 && p->precision != 64) return gm::fail(GM_EPARAM, "precision must be 32 or 64");
    if (p->nx < 3 || p->ny < 3 || p->nz < 3) return gm::fail(GM_EPARAM, "nx, ny, nz must be >= 3");
    if ((long long)p->nx * p->ny * p->nz > (1ll << 31)) return gm::fail(GM_EPARAM, "grid too large");
    if (strncmp(p->jMethod, "Stokes ", 7) != 0 && strncmp(p->jMethod, "Classic ", 8) != 0 &&
        strncmp(p->jMethod, "Stokes4th ", 10) != 0 && strncmp(p->jMethod, "StokesQuint ", 12) != 0 &&
        strncmp(p->jMethod, "StokesTri ", 10) != 0)
        return gm::fail(GM_EPARAM, "jMethod: the Stokes, Stokes4th, StokesQuint, StokesTri and Classic currents are implemented");
    if (p->pressure && strncmp(p->pMethod, "Classic ", 8) != 0) return gm::fail(GM_EPARAM, "pMethod must be Classic");
    if (p->initDistCode != 0 && p->initDistCode != 1) return gm::fail(GM_EPARAM, "initDistCode must be 0 or 1");
    if (!(p->dx > 0 && p->dy > 0 && p->dz > 0)) return gm::fail(GM_EPARAM, "dx, dy, dz must be > 0 (call gm_params_derive)");
    if (p->errMode != 0 && p->errMode != 1) return gm::fail(GM_EPARAM, "errMode must be 0 or 1");
    if (p->stageKernel != 0 && p->stageKernel != 1) return gm::fail(GM_EPARAM, "stageKernel must be 0 or 1");
    return GM_OK;
}

struct ImplBase {
    virtual ~ImplBase() {}
    virtual int upload(const void* xb, const void* B0, double t, double dt) = 0;
    virtual int stage(int n) = 0;
    virtual int control() = 0;
    virtual int steps_async(int n) = 0;
    virtual int run(int nCycle, gm_state* out) = 0;
    virtual int run_events(int nCycle, gm_state* out) = 0;
    virtual int grid_fields(void* cellVol, void* convexity, void* wedgeMin) = 0;
    virtual int get_state(gm_state* out) = 0;
    virtual int set_dt(double t, double dt, int timeIndex) = 0;
    virtual int refresh(gm_reduction* r) = 0;
    virtual int download(void* xb, void* B, void* J, void* D) = 0;
    virtual int download_k(int m, void* k) = 0;
    virtual int download_x(int which, void* xb) = 0;
    virtual int upload_u(const void* u) = 0;
    virtual int download_u(int which, void* u) = 0;
    virtual int step(gm_step_result* r) = 0;
    virtual int autotune(int trials, int* tz, double* ms) = 0;
    virtual int set_tile_z(int tz) = 0;
    virtual int debug_stall(int on) = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    int64_t launches = 0;
    bool uploaded = false;
    bool stall_on = false;   // gm_debug_stall
};

template <typename T>
struct Impl : ImplBase {
    gm_params gp;
    KP<T> kp;
    // device buffers
    T* X[2] = {nullptr, nullptr};
    T* XS[2] = {nullptr, nullptr};
    T* K[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // inertia: velocity (pitched inner SoA, as K): U[cur] at the step start,
    // US stage ping-pong, KU the velocity increments
    T* U[2] = {nullptr, nullptr};
    T* US[2] = {nullptr, nullptr};
    T* KU[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    T* B0 = nullptr;
    T* B0s = nullptr;           // B0 scaled for the algebraic B formula
    T* shear_tab = nullptr;     // initially distorted grid: the z ghost planes' corrected positions
    T* outB = nullptr;
    T* outJ = nullptr;
    T* outD = nullptr;
    T* stage_buf = nullptr;     // ghosted AoS staging for transfers
    T* eps = nullptr;           // ex | ey | ez
    T* eps_col = nullptr;       // eps* scratch: J.B/B^2 and z of the central column
    DevState* st = nullptr;
    double* log = nullptr;
    double* part = nullptr;
    double* red = nullptr;
    DevState* h_st = nullptr;   // pinned
    double* h_red = nullptr;    // pinned
    int logCap = 0;
    // launch shape
    int TY = 8, TZ = 32;
    dim3 grid, block;
    size_t smem_stage = 0, smem_diag = 0;
    int nparts = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int64_t step_launches = 7;      // kernel launches in the captured step
    // TMA-fed stage kernel: tensor maps of X[0], X[1], XS[0], XS[1]
    bool use_tma = true;
    CUtensorMap tmaps[10];      // single-case kernel (tile height stage_tma_ty<T>(pressure))
    CUtensorMap tmaps_b[10];    // batched kernel (tile height STAGE_BATCH_TY)
    dim3 grid2;
    int TZ2 = 32;
    size_t NG = 0, N = 0, NP = 0;

    ~Impl() override {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        void* ptrs[] = {X[0], X[1], XS[0], XS[1], K[0], K[1], K[2], K[3], K[4], B0, B0s, outB, outJ,
                        outD, stage_buf, eps, eps_col, st, log, part, red, U[0], U[1], US[0], US[1],
                        KU[0], KU[1], KU[2], KU[3], KU[4], shear_tab};
        for (void* q : ptrs)
            if (q) cudaFree(q);
        if (h_st) cudaFreeHost(h_st);
        if (h_red) cudaFreeHost(h_red);
        if (own_stream) cudaStreamDestroy(own_stream);
    }

    int alloc(void** pp, size_t bytes) {
        cudaError_t e = cudaMalloc(pp, bytes);
        if (e != cudaSuccess) return gm::fail(GM_EALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        e = cudaMemsetAsync(*pp, 0, bytes, stream);
        if (e != cudaSuccess) return gm::fail(GM_ECUDA, std::string("cudaMemset: ") + cudaGetErrorString(e));
        return GM_OK;
    }

    int init(const gm_params* p) {
        gp = *p;
        CUDA_TRY(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
        stream = own_stream;
        CUDA_TRY(gmk::prepare_kernels<T>());
        const int nx = p->nx, ny = p->ny, nz = p->nz;
        memset(&kp, 0, sizeof kp);
        kp.nx = nx; kp.ny = ny; kp.nz = nz;
        kp.px = ((nx + 4) + 7) / 8 * 8;
        kp.py = ny + 4;
        kp.pz = nz + 4;
        kp.cs = ((long long)kp.px * kp.py * kp.pz + 63) / 64 * 64;
        kp.N = (long long)nx * ny * nz;
        kp.kpx = (nx + 7) / 8 * 8;
        kp.kcs = ((long long)kp.kpx * ny * nz + 63) / 64 * 64;
        kp.dx = (T)p->dx; kp.dy = (T)p->dy; kp.dz = (T)p->dz;
        kp.dx1 = (T)p->dx1; kp.dy1 = (T)p->dy1; kp.dz1 = (T)p->dz1;
        kp.hdx1 = kp.dx1 / 2; kp.hdy1 = kp.dy1 / 2; kp.hdz1 = kp.dz1 / 2;
        kp.Lx = (T)p->Lx; kp.Ly = (T)p->Ly; kp.Lz = (T)p->Lz;
        kp.Ox = (T)p->Ox; kp.Oy = (T)p->Oy; kp.Oz = (T)p->Oz;
        kp.xPeri = p->xPeri != 0; kp.yPeri = p->yPeri != 0; kp.zPeri = p->zPeri != 0;
        kp.zUpdate = p->zUpdate != 0;
        kp.errMode = p->errMode;
        kp.refDt = p->errMode == 0;
        kp.jClassic = strncmp(p->jMethod, "Classic ", 8) == 0;
        kp.jOct = strncmp(p->jMethod, "Stokes4th ", 10) == 0;
        kp.jQuint = strncmp(p->jMethod, "StokesQuint ", 12) == 0;
        kp.jTri = strncmp(p->jMethod, "StokesTri ", 10) == 0;
        kp.inertia = p->inertia != 0;
        kp.nu = (T)p->nu;
        kp.jxbAver = p->jxbAver != 0 && !p->inertia;   // the reference applies it in the frictional branch only
        kp.jxbW = (T)p->jxbAverWeight;
        kp.beta = (T)p->beta;
        kp.p0Amp = (T)p->p0Amp;
        kp.p0W2 = (T)(p->p0Width * p->p0Width);
        kp.inv_p0W2 = kp.p0W2 != (T)0 ? (T)1 / kp.p0W2 : (T)0;
        kp.maxError = (double)(T)p->maxError;
        kp.dtMin = (double)(T)p->dtMin;
        kp.ar = p->ar; kp.az = p->az; kp.phi1 = p->phi1;
        kp.shear = p->initShearA != 0 || p->initShearB != 0;
        kp.initDistCode = p->initDistCode;
        kp.shA = (T)p->initShearA; kp.shB = (T)p->initShearB; kp.shK = (T)p->initShearK;
        kp.wantXbAn = p->redErrXb_XbAn != 0;
        kp.nTs = p->nTs;
        kp.dtDump = (T)p->dtDump;
        kp.dtSave = (T)p->dtSave;
        // Cash-Karp tableau, src/rungeKutta.cu:10-25
        static const double bd[7][6] = {
            {0, 0, 0, 0, 0, 0},
            {0.2, 0, 0, 0, 0, 0},
            {3 / 40., 9 / 40., 0, 0, 0, 0},
            {0.3, -0.9, 1.2, 0, 0, 0},
            {-11 / 54., 2.5, -70 / 27., 35 / 27., 0, 0},
            {1631 / 55296., 175 / 512., 575 / 13824., 44275 / 110592., 253 / 4096., 0},
            {0, 0, 0, 0, 0, 0}};
        static const double cd[6] = {37 / 378., 0, 250 / 621., 125 / 594., 0, 512 / 1771.};
        static const double csd[6] = {2825 / 27648., 0, 18575 / 48384., 13525 / 55296., 277 / 14336., 0.25};
        for (int n = 0; n < 6; n++)
            for (int m = 0; m < 6; m++) kp.db[n][m] = (T)bd[n + 1][m] - (T)bd[n][m];
        for (int m = 0; m < 6; m++) {
            kp.c[m] = (T)cd[m];
            kp.cst[m] = (T)csd[m];
            kp.cmc[m] = (double)(T)cd[m] - (double)(T)csd[m];
            kp.cmcT[m] = (T)kp.cmc[m];
        }
        kp.inv8dxdydz = (T)(1.0 / (8.0 * (double)(T)p->dx * (double)(T)p->dy * (double)(T)p->dz));
        NG = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
        N = (size_t)kp.N;
        NP = (size_t)kp.cs * 3;
        int rc;
        for (int q = 0; q < 2; q++) {
            if ((rc = alloc((void**)&X[q], NP * sizeof(T)))) return rc;
            if ((rc = alloc((void**)&XS[q], NP * sizeof(T)))) return rc;
        }
        for (int m = 0; m < 5; m++)
            if ((rc = alloc((void**)&K[m], 3 * (size_t)kp.kcs * sizeof(T)))) return rc;
        if (kp.inertia) {
            for (int q = 0; q < 2; q++) {
                if ((rc = alloc((void**)&U[q], 3 * (size_t)kp.kcs * sizeof(T)))) return rc;
                if ((rc = alloc((void**)&US[q], 3 * (size_t)kp.kcs * sizeof(T)))) return rc;
            }
            for (int m = 0; m < 5; m++)
                if ((rc = alloc((void**)&KU[m], 3 * (size_t)kp.kcs * sizeof(T)))) return rc;
        }
        if ((rc = alloc((void**)&B0, NP * sizeof(T)))) return rc;
        if ((rc = alloc((void**)&B0s, NP * sizeof(T)))) return rc;
        if (kp.shear) {
            if ((rc = alloc((void**)&shear_tab, (size_t)20 * nx * ny * sizeof(T)))) return rc;
            kp.shearTab = shear_tab;
        }
        if ((rc = alloc((void**)&outB, 3 * NG * sizeof(T)))) return rc;
        if ((rc = alloc((void**)&outJ, 3 * N * sizeof(T)))) return rc;
        if ((rc = alloc((void**)&outD, NG * sizeof(T)))) return rc;
        // ghosted AoS fields, or with inertia the 6-value k records of the inner points
        const size_t stage_elems = kp.inertia ? std::max(3 * NG, 6 * N) : 3 * NG;
        if ((rc = alloc((void**)&stage_buf, stage_elems * sizeof(T)))) return rc;
        if ((rc = alloc((void**)&eps, (size_t)(nx + ny + nz) * sizeof(T)))) return rc;
        if ((rc = alloc((void**)&eps_col, (size_t)2 * nz * sizeof(T)))) return rc;
        if ((rc = alloc((void**)&st, sizeof(DevState)))) return rc;
        logCap = 1 << 16;
        if ((rc = alloc((void**)&log, (size_t)3 * logCap * sizeof(double)))) return rc;
        CUDA_TRY(cudaMallocHost((void**)&h_st, sizeof(DevState)));
        CUDA_TRY(cudaMallocHost((void**)&h_red, (gmk::R_COUNT + 1) * sizeof(double)));
        // epsilon profile factors, src/rungeKutta.cu:180-185 (evaluated in double)
        {
            std::vector<T> e((size_t)nx + ny + nz);
            const int n3[3] = {nx, ny, nz};
            size_t o = 0;
            for (int a = 0; a < 3; a++)
                for (int i = 0; i < n3[a]; i++) {
                    const int n = n3[a];
                    e[o++] = p->epsilonProf ? (T)(-(i - n / 2.) / n * (i + 1 - n / 2.) / n * 4 + 1) : (T)1;
                }
            CUDA_TRY(cudaMemcpyAsync(eps, e.data(), e.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaStreamSynchronize(stream));
        }
        kp.ex = eps;
        kp.ey = eps + nx;
        kp.ez = eps + nx + ny;
        // launch shape: 32 x TY column tiles of TZ planes.  Pick (TY, TZ) to
        // minimise the work of the busiest SM, ceil(tiles / SMs) x per-tile
        // work (TZ + 3) x (TY + 2) (the +3 / +2 are the halo planes and rows
        // a tile recomputes), so tiles split evenly over the 152 SMs.
        const int nbx = (nx + gmk::TX - 1) / gmk::TX;
        int dev = 0, nsm = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        double best = 1e300;
        for (int ty : {8, 4, 2}) {
            if (ty > 2 && ny < ty) continue;
            const size_t sm = gmk::stage_smem_bytes<T>(ty, gmk::MODE_STAGE, p->pressure);
            const long long slots = (long long)nsm * gmk::stage_occupancy<T>(ty, p->pressure, sm);
            const long long ncol = (long long)nbx * ((ny + ty - 1) / ty);
            for (int nzc = 1; nzc <= nz; nzc++) {
                const int tz = (nz + nzc - 1) / nzc;
                if (tz < 4 && nz >= 4) break;
                const long long tiles = ncol * ((nz + tz - 1) / tz);
                const long long per_sm = (tiles + nsm - 1) / nsm;
                if (tiles < slots / 4 && ty > 2) continue;   // too few CTAs to fill the GPU
                const double cost = (double)per_sm * (tz + 3) * (ty + 2);
                if (cost < best * 0.999) { best = cost; TY = ty; TZ = tz; }
            }
        }
        grid = dim3((unsigned)nbx, (unsigned)((ny + TY - 1) / TY), (unsigned)((nz + TZ - 1) / TZ));
        block = dim3(gmk::TX, (unsigned)TY, 1);
        smem_stage = gmk::stage_smem_bytes<T>(TY, gmk::MODE_STAGE, p->pressure);
        smem_diag = gmk::stage_smem_bytes<T>(TY, gmk::MODE_DIAG, p->pressure);
        nparts = (int)(grid.x * grid.y * grid.z);
        // the TMA kernel computes the Stokes current of the frictional
        // equation only; the other currents, the inertial equation and the
        // averaged Lorentz force run in the generic kernel
        use_tma = p->stageKernel == 0 && strncmp(p->jMethod, "Stokes ", 7) == 0 && !p->inertia && !p->jxbAver;
        if (use_tma) {
            if ((rc = init_tma(nsm))) return rc;
        }
        if ((rc = alloc((void**)&part, (size_t)nparts * gmk::R_COUNT * sizeof(double)))) return rc;
        if ((rc = alloc((void**)&red, (gmk::R_COUNT + 1) * sizeof(double)))) return rc;   // + eps*
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    // Tensor maps over the padded positions viewed as (px, py, pz, component),
    // box 36 x (ty + 4) x 1 x 3 = one position plane of a 32 x ty tile with its
    // 2-point halo, and over the k arrays, box 32 x ty x 1 x 3: one set for the
    // single-case tile height, one for the batched one.  Box x starts are tile
    // starts (multiples of 32 elements), so every copy starts on a 16-byte
    // boundary.
    int init_tma(int nsm) {
        CUDA_TRY(gmk::prepare_stage_tma<T>());
        int rc = encode_maps(tmaps, gmk::stage_tma_ty<T>(gp.pressure));
        if (!rc) rc = encode_maps(tmaps_b, gmk::STAGE_BATCH_TY);
        if (rc) return rc;
        choose_tz2(nsm);
        return GM_OK;
    }

    int encode_maps(CUtensorMap* maps, int ty) {
        auto enc = tensor_map_encoder();
        if (!enc) return gm::fail(GM_ECUDA, "cuTensorMapEncodeTiled is unavailable");
        const cuuint64_t es = sizeof(T);
        cuuint64_t dims[4] = {(cuuint64_t)kp.px, (cuuint64_t)kp.py, (cuuint64_t)kp.pz, 3};
        cuuint64_t strides[3] = {(cuuint64_t)kp.px * es, (cuuint64_t)kp.px * kp.py * es, (cuuint64_t)kp.cs * es};
        cuuint32_t box[4] = {gmk::TX + 4, (cuuint32_t)ty + 4, 1, 3};
        cuuint32_t estr[4] = {1, 1, 1, 1};
        const CUtensorMapDataType dtype = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
        T* bufs[5] = {X[0], X[1], XS[0], XS[1], B0s};
        for (int q = 0; q < 5; q++) {
            CUresult r = enc(&maps[q], dtype, 4, (void*)bufs[q], dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return gm::fail(GM_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
        }
        // k_m over (nx, ny, nz, component), row pitch kpx: box 32 x 8 x 1 x 3, the tile
        // (rows start on 16-byte boundaries: kpx is a multiple of 8)
        cuuint64_t kdims[4] = {(cuuint64_t)kp.nx, (cuuint64_t)kp.ny, (cuuint64_t)kp.nz, 3};
        cuuint64_t kstrides[3] = {(cuuint64_t)kp.kpx * es, (cuuint64_t)kp.kpx * kp.ny * es, (cuuint64_t)kp.kcs * es};
        cuuint32_t kbox[4] = {gmk::TX, (cuuint32_t)ty, 1, 3};
        for (int m = 0; m < 5; m++) {
            CUresult r = enc(&maps[5 + m], dtype, 4, (void*)K[m], kdims, kstrides, kbox, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return gm::fail(GM_ECUDA, "cuTensorMapEncodeTiled (k) failed: " + std::to_string((int)r));
        }
        return GM_OK;
    }

    // z chunking of the single-case TMA kernel: minimise the iterations of the
    // busiest SM, ceil(tiles / SMs) x (TZ + 2) (the kernel is issue-bound, so
    // an SM's time follows the work of all the tiles it runs)
    void choose_tz2(int nsm) {
        const int nx = kp.nx, ny = kp.ny, nz = kp.nz;
        const int ty = gmk::stage_tma_ty<T>(gp.pressure);
        const long long ncol = (long long)((nx + gmk::TX - 1) / gmk::TX) * ((ny + ty - 1) / ty);
        double best = 1e300;
        for (int nzc = 1; nzc <= nz; nzc++) {
            const int tz = (nz + nzc - 1) / nzc;
            if (tz < 4 && nz >= 4) break;
            const long long tiles = ncol * ((nz + tz - 1) / tz);
            const long long per_sm = (tiles + nsm - 1) / nsm;
            const double cost = (double)per_sm * (tz + 2);   // tz + 2 iterations per tile
            if (cost < best * 0.999) { best = cost; TZ2 = tz; }
        }
        grid2 = dim3((unsigned)((nx + gmk::TX - 1) / gmk::TX), (unsigned)((ny + ty - 1) / ty),
                     (unsigned)((nz + TZ2 - 1) / TZ2));
    }

    StageArgs<T> args(int n) {
        StageArgs<T> a;
        memset(&a, 0, sizeof a);
        a.p = kp;
        a.X[0] = X[0]; a.X[1] = X[1];
        a.XS[0] = XS[0]; a.XS[1] = XS[1];
        for (int m = 0; m < 5; m++) a.K[m] = K[m];
        a.U[0] = U[0]; a.U[1] = U[1];
        a.US[0] = US[0]; a.US[1] = US[1];
        for (int m = 0; m < 5; m++) a.KU[m] = KU[m];
        a.B0 = B0;
        a.B0s = B0s;
        a.st = st;
        a.log = log;
        a.n = n;
        a.stall = stall_on ? 1 : 0;
        a.TZ = TZ;
        a.outB = outB; a.outJ = outJ; a.outD = outD;
        a.part = part;
        return a;
    }

    int upload(const void* xb, const void* b0, double t, double dt) override {
        if (!xb || !b0) return gm::fail(GM_EPARAM, "gm_upload: null array");
        const size_t bytes = 3 * NG * sizeof(T);
        // host or device arrays (unified addressing)
        CUDA_TRY(cudaMemcpyAsync(stage_buf, b0, bytes, cudaMemcpyDefault, stream));
        CUDA_TRY(gmk::launch_unpack<T>(kp, stage_buf, B0, stream));
        CUDA_TRY(gmk::launch_scale_b0<T>(kp, B0, B0s, stream));
        CUDA_TRY(cudaMemcpyAsync(outB, stage_buf, bytes, cudaMemcpyDeviceToDevice, stream));   // main.cu:195
        CUDA_TRY(cudaMemcpyAsync(stage_buf, xb, bytes, cudaMemcpyDefault, stream));
        T* bufs[4] = {X[0], X[1], XS[0], XS[1]};
        for (T* b : bufs) {
            CUDA_TRY(gmk::launch_unpack<T>(kp, stage_buf, b, stream));
            CUDA_TRY(gmk::launch_images<T>(kp, b, stream));
        }
        launches += 10;
        if (kp.shear) {
            // the line-tied z ghost planes of the uploaded grid, with addDist
            CUDA_TRY(gmk::launch_shear_table<T>(kp, X[0], shear_tab, stream));
            launches++;
        }
        if (kp.inertia) {
            // uInit = "nil": zero velocity (the reference allocates uu with
            // malloc and leaves it unset, memory.cu:33-35, init.cu:362-364)
            for (T* b : {U[0], U[1], US[0], US[1]})
                CUDA_TRY(cudaMemsetAsync(b, 0, 3 * (size_t)kp.kcs * sizeof(T), stream));
        }
        DevState s;
        memset(&s, 0, sizeof s);
        s.t = gp.errMode == 0 ? (double)(T)t : t;
        s.dt = gp.errMode == 0 ? (double)(T)dt : dt;
        s.target = INT_MAX;
        s.logCap = logCap;
        s.done = !(s.dt > kp.dtMin);
        if (s.done) s.status |= GM_ST_DTMIN | GM_ST_DONE;
        *h_st = s;
        CUDA_TRY(cudaMemcpyAsync(st, h_st, sizeof s, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        uploaded = true;
        ev_base = -1;
        return GM_OK;
    }

    int stage(int n) override {
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_stage before gm_upload");
        if (n < 0 || n > 5) return gm::fail(GM_EPARAM, "stage index must be 0..5");
        if (use_tma) {
            gmk::StageArgsTMA<T> A;
            memcpy(A.tm, tmaps, sizeof tmaps);
            A.a = args(n);
            A.a.TZ = TZ2;
            CUDA_TRY(gmk::launch_stage_tma<T>(A, gp.pressure, grid2, stream));
        } else {
            if (kp.jxbAver || kp.jOct || kp.jQuint || kp.jTri) {
                // the averaged Lorentz force reads J and B of this stage at every
                // point's neighbours, and the octilateral current B at the edge
                // neighbours with the reference's ghost values (current() before
                // kk(), main.cu:272-281): a J pass exports B (and J) first
                StageArgs<T> aj = args(n);
                aj.jpass = 1;
                CUDA_TRY(gmk::launch_stage<T>(aj, gmk::MODE_DIAG, gp.pressure, grid, block, smem_diag, stream));
                CUDA_TRY(gmk::launch_export_ghosts<T>(kp, outB, outD, stream));
                launches += 1 + kp.xPeri + kp.yPeri + kp.zPeri;
                if (kp.jOct || kp.jQuint || kp.jTri) {
                    CUDA_TRY(kp.jOct ? gmk::launch_j_oct<T>(args(n), stream) : gmk::launch_j_quint<T>(args(n), stream));
                    launches++;
                }
            }
            StageArgs<T> a = args(n);
            CUDA_TRY(gmk::launch_stage<T>(a, gmk::MODE_STAGE, gp.pressure, grid, block, smem_stage, stream));
        }
        launches++;
        return GM_OK;
    }

    int control() override {
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_control before gm_upload");
        CUDA_TRY(gmk::launch_control<T>(kp, st, log, stream));
        launches++;
        return GM_OK;
    }

    int enqueue_step() {
        int rc;
        for (int n = 0; n < 6; n++)
            if ((rc = stage(n))) return rc;
        return control();
    }

    int steps_async(int nsteps) override {
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_steps_async before gm_upload");
        if (nsteps <= 0) return GM_OK;
        if (!gexec) {
            // capture one attempted step on a private stream
            cudaStream_t cs;
            CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
            cudaStream_t saved = stream;
            int64_t saved_launches = launches;
            stream = cs;
            cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
            int rc = e == cudaSuccess ? enqueue_step() : GM_ECUDA;
            cudaGraph_t g = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(cs, &g);
            stream = saved;
            step_launches = launches - saved_launches;
            launches = saved_launches;
            cudaStreamDestroy(cs);
            if (e != cudaSuccess || rc != GM_OK || e2 != cudaSuccess)
                return gm::fail(GM_ECUDA, "capture of the step graph failed");
            graph = g;
            CUDA_TRY(cudaGraphInstantiate(&gexec, graph, 0));
        }
        for (int s = 0; s < nsteps; s++) {
            CUDA_TRY(cudaGraphLaunch(gexec, stream));
            launches += step_launches;
        }
        return GM_OK;
    }

    // Autotuner of the TMA stage kernel's z-chunk depth TZ2 (the tile shape in
    // z: planes a CTA marches through, each chunk paying two halo planes).
    // Candidates: the eight best depths by the cost model of choose_tz2 and
    // the current one.  Each is timed with CUDA events on the handle's stream over
    // `trials` rounds of stages 0..4 on the uploaded state (those stages write
    // only the stage buffers, not the step-start grid), after one untimed
    // round; the fastest is kept and the step graph recaptured with it.
    int autotune(int trials, int* tz_out, double* ms_out) override {
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_autotune before gm_upload");
        if (trials < 1) return gm::fail(GM_EPARAM, "gm_autotune: trials must be >= 1");
        if (!use_tma) {   // the generic kernel's tile is chosen by its own model
            if (tz_out) *tz_out = TZ;
            if (ms_out) *ms_out = 0;
            return GM_OK;
        }
        int dev = 0, nsm = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        const int nx = kp.nx, ny = kp.ny, nz = kp.nz, ty = gmk::stage_tma_ty<T>(gp.pressure);
        const long long ncol = (long long)((nx + gmk::TX - 1) / gmk::TX) * ((ny + ty - 1) / ty);
        std::vector<std::pair<double, int>> cand;
        int last = -1;
        for (int nzc = 1; nzc <= nz; nzc++) {
            const int tz = (nz + nzc - 1) / nzc;
            if (tz < 4 && nz >= 4) break;
            if (tz == last) continue;
            last = tz;
            const long long tiles = ncol * ((nz + tz - 1) / tz);
            cand.emplace_back((double)((tiles + nsm - 1) / nsm) * (tz + 2), tz);
        }
        std::sort(cand.begin(), cand.end());
        std::vector<int> tzs;
        for (size_t q = 0; q < cand.size() && tzs.size() < 8; q++) tzs.push_back(cand[q].second);
        if (std::find(tzs.begin(), tzs.end(), TZ2) == tzs.end()) tzs.push_back(TZ2);
        cudaEvent_t e0, e1;
        CUDA_TRY(cudaEventCreate(&e0));
        CUDA_TRY(cudaEventCreate(&e1));
        double best_ms = 1e300;
        int best_tz = TZ2;
        int rc = GM_OK;
        for (int tz : tzs) {
            TZ2 = tz;
            grid2 = dim3(grid2.x, grid2.y, (unsigned)((nz + tz - 1) / tz));
            for (int r = 0; r <= trials && rc == GM_OK; r++) {
                if (r == 1 && cudaEventRecord(e0, stream) != cudaSuccess) rc = GM_ECUDA;
                for (int n = 0; n < 5 && rc == GM_OK; n++) rc = stage(n);
            }
            if (rc != GM_OK) break;
            float ms = 0;
            if (cudaEventRecord(e1, stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                rc = gm::fail(GM_ECUDA, "gm_autotune: event timing failed");
                break;
            }
            if (ms < best_ms) { best_ms = ms; best_tz = tz; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        TZ2 = best_tz;
        grid2 = dim3(grid2.x, grid2.y, (unsigned)((nz + best_tz - 1) / best_tz));
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
        if (rc != GM_OK) return rc;
        if (tz_out) *tz_out = best_tz;
        if (ms_out) *ms_out = best_ms / trials;
        return GM_OK;
    }

    int debug_stall(int on) override {
        if (!use_tma) return gm::fail(GM_EPARAM, "gm_debug_stall: the run does not use the TMA stage kernel");
        stall_on = on != 0;
        // the step graph holds the launch arguments: capture it again
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
        return GM_OK;
    }

    int set_tile_z(int tz) override {
        if (!use_tma) return gm::fail(GM_EPARAM, "gm_set_tile_z: the run does not use the TMA stage kernel");
        if (tz < 1 || tz > kp.nz) return gm::fail(GM_EPARAM, "gm_set_tile_z: depth must be 1..nz");
        TZ2 = tz;
        grid2 = dim3(grid2.x, grid2.y, (unsigned)((kp.nz + tz - 1) / tz));
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
        return GM_OK;
    }

    int read_state() {
        CUDA_TRY(cudaMemcpyAsync(h_st, st, sizeof(DevState), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    void fill(gm_state* o) {
        o->t = h_st->t;
        o->dt = h_st->dt;
        o->maxDelta = h_st->maxDelta;
        o->timeIndex = h_st->timeIndex;
        o->nAttempted = h_st->nAttempted;
        o->nRejected = h_st->nRejected;
        o->status = h_st->status;
        o->dtUsed = h_st->dtUsed;
        o->event = h_st->event;
        o->pad = 0;
    }

    int get_state(gm_state* out) override {
        int rc = read_state();
        if (rc) return rc;
        if (out) fill(out);
        return GM_OK;
    }

    int set_control(int target, bool reset_done, bool events = false) {
        int rc = read_state();
        if (rc) return rc;
        h_st->target = target;
        h_st->eventsOn = events ? 1 : 0;
        h_st->status &= ~(unsigned)GM_ST_EVENT;
        if (reset_done) {
            const bool dtmin = !(h_st->dt > kp.dtMin);
            h_st->done = dtmin || (h_st->status & (GM_ST_NAN | GM_ST_TIMEOUT | GM_ST_ALIGN)) || h_st->timeIndex >= target;
            if (dtmin) h_st->status |= GM_ST_DTMIN;
            if (h_st->done) h_st->status |= GM_ST_DONE;
            else h_st->status &= ~(unsigned)GM_ST_DONE;
        }
        CUDA_TRY(cudaMemcpyAsync(st, h_st, sizeof(DevState), cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    int set_dt(double t, double dt, int timeIndex) override {
        int rc = read_state();
        if (rc) return rc;
        h_st->t = gp.errMode == 0 ? (double)(T)t : t;
        h_st->dt = gp.errMode == 0 ? (double)(T)dt : dt;
        h_st->timeIndex = timeIndex;
        h_st->done = !(h_st->dt > kp.dtMin);
        ev_base = -1;
        CUDA_TRY(cudaMemcpyAsync(st, h_st, sizeof(DevState), cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    int run(int nCycle, gm_state* out) override {
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_run before gm_upload");
        int rc = read_state();
        if (rc) return rc;
        const long long tgt = (long long)h_st->timeIndex + nCycle;
        if ((rc = set_control(tgt > INT_MAX ? INT_MAX : (int)tgt, true))) return rc;
        // graph replays in chunks; steps after the stop rule do no work
        int chunk = 16;
        while (!h_st->done) {
            if ((rc = steps_async(chunk))) return rc;
            if ((rc = read_state())) return rc;
            if (chunk < 256) chunk *= 2;
        }
        if (out) fill(out);
        if (h_st->status & GM_ST_NAN) return gm::fail(GM_ENAN, "NaN/Inf in a stage increment");
        if (h_st->status & (GM_ST_TIMEOUT | GM_ST_ALIGN))
            return gm::fail(GM_ETIMEOUT, "a stage kernel stopped: bounded wait or alignment check (status " +
                                             std::to_string(h_st->status) + ")");
        return GM_OK;
    }

    // As run, with a stop after every accepted step whose output is due; the
    // step count is measured from the first call after upload / set_dt.
    int ev_base = -1;
    int run_events(int nCycle, gm_state* out) override {
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_run_events before gm_upload");
        if (nCycle < 0) return gm::fail(GM_EPARAM, "gm_run_events: nCycle < 0");
        int rc = read_state();
        if (rc) return rc;
        if (ev_base < 0) ev_base = h_st->timeIndex;
        const long long tgt = (long long)ev_base + nCycle;
        if ((rc = set_control(tgt > INT_MAX ? INT_MAX : (int)tgt, true, true))) return rc;
        int chunk = 1;
        while (!h_st->done) {
            if ((rc = steps_async(chunk))) return rc;
            if ((rc = read_state())) return rc;
            if (chunk < 64) chunk *= 2;
        }
        if (out) {
            fill(out);
            if (!(h_st->status & GM_ST_EVENT)) out->event = 0;
        }
        if (h_st->status & GM_ST_NAN) return gm::fail(GM_ENAN, "NaN/Inf in a stage increment");
        if (h_st->status & (GM_ST_TIMEOUT | GM_ST_ALIGN))
            return gm::fail(GM_ETIMEOUT, "a stage kernel stopped: bounded wait or alignment check (status " +
                                             std::to_string(h_st->status) + ")");
        return GM_OK;
    }

    int grid_fields(void* cellVol, void* convexity, void* wedgeMin) override {
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_grid_fields before gm_upload");
        int rc = read_state();
        if (rc) return rc;
        T* cv = stage_buf;
        T* cx = stage_buf + N;
        T* wm = stage_buf + 2 * N;
        CUDA_TRY(gmk::launch_grid_fields<T>(kp, X[h_st->cur], cv, cx, wm, stream));
        launches++;
        if (cellVol) CUDA_TRY(cudaMemcpyAsync(cellVol, cv, N * sizeof(T), cudaMemcpyDeviceToHost, stream));
        if (convexity) CUDA_TRY(cudaMemcpyAsync(convexity, cx, N * sizeof(T), cudaMemcpyDeviceToHost, stream));
        if (wedgeMin) CUDA_TRY(cudaMemcpyAsync(wedgeMin, wm, N * sizeof(T), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    int refresh(gm_reduction* r) override {
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_refresh before gm_upload");
        int rc = read_state();
        if (rc) return rc;
        StageArgs<T> a = args(0);
        if (kp.jOct || kp.jQuint || kp.jTri) {
            // the octilateral and quintilateral currents need the exported B
            // with its ghosts first; the diagnostic pass then reads J from it
            StageArgs<T> aj = args(0);
            aj.jpass = 1;
            CUDA_TRY(gmk::launch_stage<T>(aj, gmk::MODE_DIAG, gp.pressure, grid, block, smem_diag, stream));
            CUDA_TRY(gmk::launch_export_ghosts<T>(kp, outB, outD, stream));
            CUDA_TRY(kp.jOct ? gmk::launch_j_oct<T>(aj, stream) : gmk::launch_j_quint<T>(aj, stream));
            launches += 2 + kp.xPeri + kp.yPeri + kp.zPeri;
        }
        CUDA_TRY(gmk::launch_stage<T>(a, gmk::MODE_DIAG, gp.pressure, grid, block, smem_diag, stream));
        CUDA_TRY(gmk::launch_finalize<T>(part, nparts, red, stream));
        CUDA_TRY(gmk::launch_export_ghosts<T>(kp, outB, outD, stream));
        CUDA_TRY(gmk::launch_eps_star<T>(kp, outB, outJ, X[h_st->cur], eps_col, red + gmk::R_COUNT, stream));
        launches += 3 + kp.xPeri + kp.yPeri + kp.zPeri;
        CUDA_TRY(cudaMemcpyAsync(h_red, red, (gmk::R_COUNT + 1) * sizeof(double), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        reduction_from_host(r);
        return GM_OK;
    }

    // The batched run's convergence check of this case, enqueued on `stream`
    // without waiting: the diagnostic pass and its reductions, then the
    // reductions and the controller state copied to the pinned host buffers.
    // After the stream has synchronised, h_st holds the state and
    // reduction_from_host the reductions (no exported ghosts or epsilon*).
    int enqueue_check() {
        StageArgs<T> a = args(0);
        CUDA_TRY(gmk::launch_stage<T>(a, gmk::MODE_DIAG, gp.pressure, grid, block, smem_diag, stream));
        CUDA_TRY(gmk::launch_finalize<T>(part, nparts, red, stream));
        launches += 2;
        CUDA_TRY(cudaMemcpyAsync(h_red, red, (gmk::R_COUNT + 1) * sizeof(double), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaMemcpyAsync(h_st, st, sizeof(DevState), cudaMemcpyDeviceToHost, stream));
        return GM_OK;
    }

    void reduction_from_host(gm_reduction* r) const {
        if (!r) return;
        {
            const double* v = h_red;
            r->B2 = v[gmk::R_SUM_B2W] * gp.dx * gp.dy * gp.dz;
            r->residual = v[gmk::R_SUM_JB] > 0 ? v[gmk::R_SUM_CROSS] / v[gmk::R_SUM_JB] : 0.0;
            r->residualPw = v[gmk::R_SUM_PW] / (double)N;
            r->BMax = v[gmk::R_MAX_B];
            r->JMax = v[gmk::R_MAX_J];
            r->JxB_B2Max = v[gmk::R_MAX_JXBB2];
            r->minDetJac = v[gmk::R_MIN_DET];
            r->wedgeMin = v[gmk::R_MIN_WEDGE];
            r->convex = v[gmk::R_MIN_CONVEX];
            r->errB_1ez = sqrt(v[gmk::R_SUM_E1]) / sqrt((double)N);
            r->errXb_XbAn = sqrt(v[gmk::R_SUM_E2]) / sqrt((double)N);
            r->epsilonStar = v[gmk::R_COUNT];
            r->U2 = v[gmk::R_SUM_U2] * gp.dx * gp.dy * gp.dz;
            r->UMax = v[gmk::R_MAX_U];
        }
    }

    int download(void* xb, void* B, void* J, void* D) override {
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_download before gm_upload");
        if (xb) {
            int rc = read_state();
            if (rc) return rc;
            CUDA_TRY(gmk::launch_pack<T>(kp, X[h_st->cur], stage_buf, stream));
            launches++;
            CUDA_TRY(cudaMemcpyAsync(xb, stage_buf, 3 * NG * sizeof(T), cudaMemcpyDeviceToHost, stream));
        }
        if (B) CUDA_TRY(cudaMemcpyAsync(B, outB, 3 * NG * sizeof(T), cudaMemcpyDeviceToHost, stream));
        if (J) CUDA_TRY(cudaMemcpyAsync(J, outJ, 3 * N * sizeof(T), cudaMemcpyDeviceToHost, stream));
        if (D) CUDA_TRY(cudaMemcpyAsync(D, outD, NG * sizeof(T), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    int step(gm_step_result* r) override {
        int rc = enqueue_step();
        if (rc) return rc;
        if ((rc = read_state())) return rc;
        if (r) {
            r->maxDelta = h_st->maxDelta;
            r->t = h_st->t;
            r->dt = h_st->dt;
            r->accepted = h_st->lastAccepted;
            r->timeIndex = h_st->timeIndex;
            r->status = h_st->status;
            r->pad = 0;
        }
        return GM_OK;
    }

    int download_k(int m, void* k) override {
        if (m < 0 || m > 4 || !k) return gm::fail(GM_EPARAM, "gm_download_k: m must be 0..4");
        if (!kp.inertia) {
            CUDA_TRY(gmk::launch_pack_k<T>(kp, K[m], stage_buf, stream));
            launches++;
            CUDA_TRY(cudaMemcpyAsync(k, stage_buf, 3 * N * sizeof(T), cudaMemcpyDeviceToHost, stream));
        } else {
            // six values per point, the reference's kk record: k_x then k_u
            CUDA_TRY(gmk::launch_pack_k6<T>(kp, K[m], KU[m], stage_buf, stream));
            launches++;
            CUDA_TRY(cudaMemcpyAsync(k, stage_buf, 6 * N * sizeof(T), cudaMemcpyDeviceToHost, stream));
        }
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    int upload_u(const void* u) override {
        if (!kp.inertia) return gm::fail(GM_EPARAM, "gm_upload_u: the run has no velocity (inertia = F)");
        if (!uploaded) return gm::fail(GM_ENOTREADY, "gm_upload_u before gm_upload");
        if (!u) return gm::fail(GM_EPARAM, "gm_upload_u: null array");
        int rc = read_state();
        if (rc) return rc;
        CUDA_TRY(cudaMemcpyAsync(stage_buf, u, 3 * N * sizeof(T), cudaMemcpyHostToDevice, stream));
        CUDA_TRY(gmk::launch_unpack_k<T>(kp, stage_buf, U[h_st->cur], stream));
        launches++;
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    int download_u(int which, void* u) override {
        if (!kp.inertia) return gm::fail(GM_EPARAM, "gm_download_u: the run has no velocity (inertia = F)");
        if (which < 0 || which > 6 || !u) return gm::fail(GM_EPARAM, "gm_download_u: which must be 0..6");
        int rc = read_state();
        if (rc) return rc;
        const int cur = h_st->cur;
        const T* src = which <= 4 ? US[which & 1] : (which == 5 ? U[cur] : U[cur ^ 1]);
        CUDA_TRY(gmk::launch_pack_k<T>(kp, src, stage_buf, stream));
        launches++;
        CUDA_TRY(cudaMemcpyAsync(u, stage_buf, 3 * N * sizeof(T), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    int download_x(int which, void* xb) override {
        if (which < 0 || which > 6 || !xb) return gm::fail(GM_EPARAM, "gm_download_x: which must be 0..6");
        int rc = read_state();
        if (rc) return rc;
        const int cur = h_st->cur;
        T* src = which <= 4 ? XS[which & 1] : (which == 5 ? X[cur] : X[cur ^ 1]);
        CUDA_TRY(gmk::launch_pack<T>(kp, src, stage_buf, stream));
        launches++;
        CUDA_TRY(cudaMemcpyAsync(xb, stage_buf, 3 * NG * sizeof(T), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }
};

// ---- many cases in one launch per stage ------------------------------------
struct BatchBase {
    virtual ~BatchBase() {}
    virtual int upload(int c, const void* xb, const void* B0, double t, double dt) = 0;
    virtual int steps_async(int n) = 0;
    virtual int get_state(int c, gm_state* out) = 0;
    virtual int refresh(int c, gm_reduction* r) = 0;
    virtual int download(int c, void* xb, void* B, void* J, void* D) = 0;
    virtual int stop(int c) = 0;
    virtual int run(int nCycle, double residual, int pointwise, int checkEvery, gm_batch_case* out) = 0;
    virtual int autotune(int trials, int* tzb, double* ms) = 0;
    int ncases = 0;
    int64_t launches = 0;
};

template <typename T>
struct Batch : BatchBase {
    int TZB = 32;                           // planes per work item (gm_batch_autotune)
    std::vector<std::unique_ptr<Impl<T>>> cs;
    std::vector<StageArgsTMA<T>> hcases;    // host copy of d_cases
    std::vector<gm_params> params;
    cudaStream_t stream = nullptr;
    StageArgsTMA<T>* d_cases = nullptr;
    int4* d_work = nullptr;
    size_t work_cap = 0;                    // int4 entries d_work holds
    int* d_counters = nullptr;
    int nwork = 0, nblocks = 0, pressure = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;

    ~Batch() override {
        if (stream) cudaStreamSynchronize(stream);
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        if (d_cases) cudaFree(d_cases);
        if (d_work) cudaFree(d_work);
        if (d_counters) cudaFree(d_counters);
        cs.clear();
        if (stream) cudaStreamDestroy(stream);
    }

    int init(const gm_params* ps, int n) {
        ncases = n;
        pressure = ps[0].pressure != 0;
        for (int c = 0; c < n; c++)
            if ((ps[c].pressure != 0) != (pressure != 0) || ps[c].precision != ps[0].precision)
                return gm::fail(GM_EPARAM, "gm_batch_create: all cases need the same precision and pressure flag");
        CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        hcases.resize(n);
        params.assign(ps, ps + n);
        std::vector<StageArgsTMA<T>>& h = hcases;
        for (int c = 0; c < n; c++) {
            gm_params p = ps[c];
            p.stageKernel = 0;
            int rc = check_params(&p);
            if (rc) return rc;
            if (strncmp(p.jMethod, "Stokes ", 7) != 0 || p.inertia || p.jxbAver)
                return gm::fail(GM_EPARAM, "gm_batch_create: batched cases use the frictional equation and the Stokes current");
            cs.emplace_back(new Impl<T>());
            if ((rc = cs.back()->init(&p))) return rc;
            cs.back()->stream = stream;
            memcpy(h[c].tm, cs.back()->tmaps_b, sizeof h[c].tm);
            h[c].a = cs.back()->args(0);
        }
        CUDA_TRY(cudaMalloc((void**)&d_cases, n * sizeof(StageArgsTMA<T>)));
        CUDA_TRY(cudaMalloc((void**)&d_counters, 8 * sizeof(int)));
        CUDA_TRY(cudaMemsetAsync(d_counters, 0, 8 * sizeof(int), stream));
        int rc = set_work(TZB);
        if (rc) return rc;
        int dev = 0, nsm = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        nblocks = nsm * gmk::stage_tma_batch_occupancy<T>(pressure);
        return GM_OK;
    }

    // Work items of depth tzb planes, largest cases first, of every case or
    // only of the cases in *only; the cases' TZ and the device copies follow.
    int set_work(int tzb, const std::vector<int>* only = nullptr) {
        TZB = tzb;
        std::vector<std::pair<long long, int>> order;
        for (int c = 0; c < ncases; c++) {
            hcases[c].a.TZ = TZB;
            const gm_params& p = params[c];
            if (!only || std::find(only->begin(), only->end(), c) != only->end())
                order.emplace_back(-(long long)p.nx * p.ny * p.nz, c);
        }
        std::sort(order.begin(), order.end());
        std::vector<int4> work;
        for (auto& o : order) {
            const gm_params& p = params[o.second];
            const int nbx = (p.nx + gmk::TX - 1) / gmk::TX, nby = (p.ny + gmk::STAGE_BATCH_TY - 1) / gmk::STAGE_BATCH_TY;
            const int nbz = (p.nz + TZB - 1) / TZB;
            for (int bz = 0; bz < nbz; bz++)
                for (int by = 0; by < nby; by++)
                    for (int bx = 0; bx < nbx; bx++) work.push_back(make_int4(o.second, bx, by, bz));
        }
        CUDA_TRY(cudaStreamSynchronize(stream));
        nwork = (int)work.size();
        if (work.size() > work_cap) {
            // reallocated only when the list outgrows it (during a run the
            // list shrinks as cases finish)
            if (d_work) CUDA_TRY(cudaFree(d_work));
            d_work = nullptr;
            work_cap = 0;
            CUDA_TRY(cudaMalloc((void**)&d_work, work.size() * sizeof(int4)));
            work_cap = work.size();
        }
        CUDA_TRY(cudaMemcpyAsync(d_cases, hcases.data(), ncases * sizeof(StageArgsTMA<T>), cudaMemcpyHostToDevice,
                                 stream));
        CUDA_TRY(cudaMemcpyAsync(d_work, work.data(), work.size() * sizeof(int4), cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
        return GM_OK;
    }

    // Autotuner of the work-item depth (planes per tile): each candidate is
    // timed with CUDA events over `trials` rounds of the batched stages 0..4
    // (which write only the cases' stage buffers), after one untimed round.
    // The timing has every case active; as cases finish, fewer and larger
    // items balance worse, so the smallest depth within 3 % of the fastest is
    // kept.
    int autotune(int trials, int* tzb_out, double* ms_out) override {
        if (!uploaded_all()) return gm::fail(GM_ENOTREADY, "gm_batch_autotune before every case is uploaded");
        if (trials < 1) return gm::fail(GM_EPARAM, "gm_batch_autotune: trials must be >= 1");
        cudaEvent_t e0, e1;
        CUDA_TRY(cudaEventCreate(&e0));
        CUDA_TRY(cudaEventCreate(&e1));
        double best_ms = 1e300;
        int best = TZB, rc = GM_OK;
        double t_of[3] = {0, 0, 0};
        const int cands[3] = {16, 32, 64};
        for (int ci = 0; ci < 3; ci++) {
            const int tzb = cands[ci];
            if ((rc = set_work(tzb))) break;
            for (int r = 0; r <= trials && rc == GM_OK; r++) {
                if (r == 1 && cudaEventRecord(e0, stream) != cudaSuccess) rc = GM_ECUDA;
                for (int n = 0; n < 5 && rc == GM_OK; n++) {
                    if (cudaMemsetAsync(d_counters + n, 0, sizeof(int), stream) != cudaSuccess ||
                        gmk::launch_stage_tma_batch<T>(d_cases, d_work, nwork, d_counters + n, n, pressure, nblocks,
                                                       stream) != cudaSuccess)
                        rc = gm::fail(GM_ECUDA, "gm_batch_autotune: launch failed");
                }
            }
            if (rc != GM_OK) break;
            float ms = 0;
            if (cudaEventRecord(e1, stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                rc = gm::fail(GM_ECUDA, "gm_batch_autotune: event timing failed");
                break;
            }
            t_of[ci] = ms;
            if (ms < best_ms) best_ms = ms;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        const double fastest = best_ms;
        for (int ci = 2; ci >= 0; ci--)
            if (rc == GM_OK && t_of[ci] > 0 && t_of[ci] <= 1.03 * fastest) { best = cands[ci]; best_ms = t_of[ci]; }
        const int rc2 = set_work(best);
        if (cudaMemsetAsync(d_counters, 0, 8 * sizeof(int), stream) != cudaSuccess && rc == GM_OK) rc = GM_ECUDA;
        if (rc != GM_OK) return rc;
        if (rc2 != GM_OK) return rc2;
        if (tzb_out) *tzb_out = best;
        if (ms_out) *ms_out = best_ms / trials;
        return GM_OK;
    }

    bool uploaded_all() const {
        for (auto& c : cs)
            if (!c->uploaded) return false;
        return true;
    }

    int enqueue_step(cudaStream_t s) {
        for (int n = 0; n < 6; n++)
            CUDA_TRY(gmk::launch_stage_tma_batch<T>(d_cases, d_work, nwork, d_counters + n, n, pressure, nblocks, s));
        CUDA_TRY(gmk::launch_control_batch<T>(d_cases, ncases, d_counters, s));
        return GM_OK;
    }

    int upload(int c, const void* xb, const void* B0, double t, double dt) override {
        if (c < 0 || c >= ncases) return gm::fail(GM_EPARAM, "gm_batch_upload: case index out of range");
        return cs[c]->upload(xb, B0, t, dt);
    }

    int steps_async(int nsteps) override {
        if (!uploaded_all()) return gm::fail(GM_ENOTREADY, "gm_batch_steps_async before every case is uploaded");
        if (nsteps <= 0) return GM_OK;
        if (!gexec) {
            cudaStream_t cap;
            CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
            int rc = e == cudaSuccess ? enqueue_step(cap) : GM_ECUDA;
            cudaGraph_t g = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(cap, &g);
            cudaStreamDestroy(cap);
            if (e != cudaSuccess || rc != GM_OK || e2 != cudaSuccess)
                return gm::fail(GM_ECUDA, "capture of the batch step graph failed");
            graph = g;
            CUDA_TRY(cudaGraphInstantiate(&gexec, graph, 0));
        }
        for (int q = 0; q < nsteps; q++) {
            CUDA_TRY(cudaGraphLaunch(gexec, stream));
            launches += 7;
        }
        return GM_OK;
    }

    int check_case(int c, const char* what) {
        if (c < 0 || c >= ncases) return gm::fail(GM_EPARAM, std::string(what) + ": case index out of range");
        return GM_OK;
    }

    int get_state(int c, gm_state* out) override {
        int rc = check_case(c, "gm_batch_get_state");
        return rc ? rc : cs[c]->get_state(out);
    }
    int refresh(int c, gm_reduction* r) override {
        int rc = check_case(c, "gm_batch_refresh");
        return rc ? rc : cs[c]->refresh(r);
    }
    int download(int c, void* xb, void* B, void* J, void* D) override {
        int rc = check_case(c, "gm_batch_download");
        return rc ? rc : cs[c]->download(xb, B, J, D);
    }
    int stop(int c) override {
        int rc = check_case(c, "gm_batch_stop");
        if (rc) return rc;
        Impl<T>& im = *cs[c];
        if ((rc = im.read_state())) return rc;
        im.h_st->done = 1;
        im.h_st->status |= GM_ST_DONE;
        CUDA_TRY(cudaMemcpyAsync(im.st, im.h_st, sizeof(DevState), cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return GM_OK;
    }

    // Work items of the cases in `cases` at depth tzb.
    long long count_items(int tzb, const std::vector<int>& cases) const {
        long long n = 0;
        for (int c : cases) {
            const gm_params& p = params[c];
            n += (long long)((p.nx + gmk::TX - 1) / gmk::TX) * ((p.ny + gmk::STAGE_BATCH_TY - 1) / gmk::STAGE_BATCH_TY) *
                 ((p.nz + tzb - 1) / tzb);
        }
        return n;
    }

    int run(int nCycle, double residual, int pointwise, int checkEvery, gm_batch_case* out) override {
        if (!uploaded_all()) return gm::fail(GM_ENOTREADY, "gm_batch_run before every case is uploaded");
        if (checkEvery < 1 || nCycle < 0) return gm::fail(GM_EPARAM, "gm_batch_run: checkEvery >= 1, nCycle >= 0");
        int rc = run_pending(nCycle, residual, pointwise, checkEvery, out);
        // the full work list at the depth the run started with, for later steps
        const int rc2 = set_work(tuned_tzb);
        return rc ? rc : rc2;
    }

    int tuned_tzb = 32;

    int run_pending(int nCycle, double residual, int pointwise, int checkEvery, gm_batch_case* out) {
        int rc;
        tuned_tzb = TZB;
        for (int c = 0; c < ncases; c++) {
            Impl<T>& im = *cs[c];
            if ((rc = im.read_state())) return rc;
            const long long tgt = (long long)im.h_st->timeIndex + nCycle;
            if ((rc = im.set_control(tgt > INT_MAX ? INT_MAX : (int)tgt, true))) return rc;
        }
        std::vector<int> pending;
        for (int c = 0; c < ncases; c++) pending.push_back(c);
        CUDA_TRY(cudaStreamSynchronize(stream));
        const auto t0 = std::chrono::steady_clock::now();
        auto record = [&](int c, double res, bool conv, double sec) {
            if (!out) return;
            gm_state s;
            cs[c]->fill(&s);
            out[c].seconds = sec;
            out[c].residual = res;
            out[c].t = s.t;
            out[c].dt = s.dt;
            out[c].attempted = s.nAttempted;
            out[c].accepted = s.timeIndex;
            out[c].status = s.status;
            out[c].converged = conv ? 1 : 0;
        };
        while (!pending.empty()) {
            if ((rc = steps_async(checkEvery))) return rc;
            // every running case's check on the batch stream, one wait for all
            for (int c : pending)
                if ((rc = cs[c]->enqueue_check())) return rc;
            CUDA_TRY(cudaStreamSynchronize(stream));
            const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            std::vector<int> still;
            for (int c : pending) {
                Impl<T>& im = *cs[c];
                const bool done = im.h_st->done != 0;
                gm_reduction r;
                im.reduction_from_host(&r);
                const double res = pointwise ? r.residualPw : r.residual;
                const bool conv = res <= residual;
                if (conv && !done && (rc = stop(c))) return rc;
                if (conv || done) {
                    // a finished case's state and exported fields (with their
                    // ghosts), as gm_batch_refresh leaves them
                    if ((rc = im.refresh(nullptr))) return rc;
                    record(c, res, conv, sec);
                } else {
                    still.push_back(c);
                }
            }
            // As cases finish, the work list keeps only the running ones (no
            // CTA spends a claim on a stopped case), and where the depth the
            // run started with would leave fewer than two items per resident
            // CTA, 16-plane items spread the remaining cases over the SMs.
            // The depth does not change any result.
            if (!still.empty() && still.size() < pending.size()) {
                int tz = tuned_tzb;
                if (tz > 16 && count_items(tz, still) < 2LL * nblocks) tz = 16;
                if ((rc = set_work(tz, &still))) return rc;
            }
            pending.swap(still);
        }
        return GM_OK;
    }
};

}  // namespace

struct gm_handle {
    std::unique_ptr<ImplBase> impl;
    int precision;
};

struct gm_batch {
    std::unique_ptr<BatchBase> impl;
};

extern "C" {

int gm_create(const gm_params* p, gm_handle** out) {
    if (!out) return gm::fail(GM_EPARAM, "gm_create: null output");
    *out = nullptr;
    int rc = check_params(p);
    if (rc) return rc;
    gm_handle* h = new gm_handle();
    h->precision = p->precision;
    if (p->precision == 32) {
        auto* im = new Impl<float>();
        h->impl.reset(im);
        rc = im->init(p);
    } else {
        auto* im = new Impl<double>();
        h->impl.reset(im);
        rc = im->init(p);
    }
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return GM_OK;
}

int gm_destroy(gm_handle* h) {
    if (!h) return GM_OK;
    if (h->impl && h->impl->stream) cudaStreamSynchronize(h->impl->stream);
    delete h;
    return GM_OK;
}

int gm_set_stream(gm_handle* h, void* stream) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    h->impl->stream = stream ? (cudaStream_t)stream : h->impl->own_stream;
    return GM_OK;
}

int gm_upload(gm_handle* h, const void* xb, const void* B0, double t, double dt) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->upload(xb, B0, t, dt);
}

int gm_stage(gm_handle* h, int n) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->stage(n);
}

int gm_control(gm_handle* h) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->control();
}

int gm_step(gm_handle* h, gm_step_result* r) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->step(r);
}

int gm_steps_async(gm_handle* h, int nSteps) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->steps_async(nSteps);
}

int gm_run(gm_handle* h, int nCycle, gm_state* out) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->run(nCycle, out);
}

int gm_run_events(gm_handle* h, int nCycle, gm_state* out) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->run_events(nCycle, out);
}

int gm_debug_stall(gm_handle* h, int on) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->debug_stall(on);
}

int gm_grid_fields(gm_handle* h, void* cellVol, void* convexity, void* wedgeMin) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->grid_fields(cellVol, convexity, wedgeMin);
}

int gm_get_state(gm_handle* h, gm_state* out) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->get_state(out);
}

int gm_set_dt(gm_handle* h, double t, double dt, int timeIndex) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->set_dt(t, dt, timeIndex);
}

int gm_refresh(gm_handle* h, gm_reduction* r) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->refresh(r);
}

int gm_download(gm_handle* h, void* xb, void* B, void* J, void* detJac) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->download(xb, B, J, detJac);
}

int gm_upload_u(gm_handle* h, const void* u) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->upload_u(u);
}

int gm_download_u(gm_handle* h, int which, void* u) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->download_u(which, u);
}

int gm_set_tile_z(gm_handle* h, int tz) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->set_tile_z(tz);
}

int gm_autotune(gm_handle* h, int trials, int* tz, double* ms) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->autotune(trials, tz, ms);
}

int gm_download_k(gm_handle* h, int m, void* k) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->download_k(m, k);
}

int gm_download_x(gm_handle* h, int which, void* xb) {
    if (!h) return gm::fail(GM_EPARAM, "null handle");
    return h->impl->download_x(which, xb);
}

int64_t gm_launch_count(const gm_handle* h) { return h ? h->impl->launches : 0; }

int gm_batch_create(const gm_params* cases, int nCases, gm_batch** out) {
    if (!out || !cases || nCases < 1) return gm::fail(GM_EPARAM, "gm_batch_create: need cases and an output");
    *out = nullptr;
    gm_batch* b = new gm_batch();
    int rc;
    if (cases[0].precision == 32) {
        auto* im = new Batch<float>();
        b->impl.reset(im);
        rc = im->init(cases, nCases);
    } else {
        auto* im = new Batch<double>();
        b->impl.reset(im);
        rc = im->init(cases, nCases);
    }
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return GM_OK;
}

int gm_batch_autotune(gm_batch* b, int trials, int* tzb, double* ms) {
    if (!b) return gm::fail(GM_EPARAM, "null batch");
    return b->impl->autotune(trials, tzb, ms);
}

int gm_batch_destroy(gm_batch* b) {
    delete b;
    return GM_OK;
}

int gm_batch_upload(gm_batch* b, int c, const void* xb, const void* B0, double t, double dt) {
    if (!b) return gm::fail(GM_EPARAM, "null batch");
    return b->impl->upload(c, xb, B0, t, dt);
}

int gm_batch_steps_async(gm_batch* b, int nSteps) {
    if (!b) return gm::fail(GM_EPARAM, "null batch");
    return b->impl->steps_async(nSteps);
}

int gm_batch_get_state(gm_batch* b, int c, gm_state* out) {
    if (!b) return gm::fail(GM_EPARAM, "null batch");
    return b->impl->get_state(c, out);
}

int gm_batch_refresh(gm_batch* b, int c, gm_reduction* r) {
    if (!b) return gm::fail(GM_EPARAM, "null batch");
    return b->impl->refresh(c, r);
}

int gm_batch_download(gm_batch* b, int c, void* xb, void* B, void* J, void* detJac) {
    if (!b) return gm::fail(GM_EPARAM, "null batch");
    return b->impl->download(c, xb, B, J, detJac);
}

int gm_batch_stop(gm_batch* b, int c) {
    if (!b) return gm::fail(GM_EPARAM, "null batch");
    return b->impl->stop(c);
}

int gm_batch_run(gm_batch* b, int nCycle, double residual, int pointwise, int checkEvery, gm_batch_case* out) {
    if (!b) return gm::fail(GM_EPARAM, "null batch");
    return b->impl->run(nCycle, residual, pointwise, checkEvery, out);
}

int64_t gm_batch_launch_count(const gm_batch* b) { return b ? b->impl->launches : 0; }


}  // extern "C"
