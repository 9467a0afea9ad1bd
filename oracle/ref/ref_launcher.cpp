// ref_launcher.cpp -- ORACLE: test infrastructure only.
//
// Drives the reference's own CUDA kernels (oracle/_ref/glemur_ref{32,64}.cubin,
// compiled unchanged from the reference sources) with the launch sequence of
// the reference host driver src/main.cu:259-384: the same kernels, block and
// grid shapes, dynamic shared-memory sizes, launch order and device
// synchronisations, the device-to-device copies, and the host-looped global
// maximum findDevMax (src/maths.cu:101-130).  Used to produce the golden
// fixtures that pin the CPU oracle, and to time the reference build.
//
// The CUDA driver API is reached through dlopen so the library builds without
// a GPU or a link-time libcuda.
#include <cuda.h>
#include <dlfcn.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/glemur.h"

namespace {

// ---- driver API entry points ----------------------------------------------
struct Drv {
    void* lib = nullptr;
    CUresult (*Init)(unsigned);
    CUresult (*DeviceGet)(CUdevice*, int);
    CUresult (*DevicePrimaryCtxRetain)(CUcontext*, CUdevice);
    CUresult (*DevicePrimaryCtxRelease)(CUdevice);
    CUresult (*CtxSetCurrent)(CUcontext);
    CUresult (*CtxSynchronize)(void);
    CUresult (*ModuleLoad)(CUmodule*, const char*);
    CUresult (*ModuleUnload)(CUmodule);
    CUresult (*ModuleGetFunction)(CUfunction*, CUmodule, const char*);
    CUresult (*ModuleGetGlobal)(CUdeviceptr*, size_t*, CUmodule, const char*);
    CUresult (*MemAlloc)(CUdeviceptr*, size_t);
    CUresult (*MemFree)(CUdeviceptr);
    CUresult (*MemsetD8)(CUdeviceptr, unsigned char, size_t);
    CUresult (*MemcpyHtoD)(CUdeviceptr, const void*, size_t);
    CUresult (*MemcpyDtoH)(void*, CUdeviceptr, size_t);
    CUresult (*MemcpyDtoD)(CUdeviceptr, CUdeviceptr, size_t);
    CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                             CUstream, void**, void**);
    CUresult (*GetErrorString)(CUresult, const char**);
};
Drv D;
std::string g_err;

template <typename F>
bool sym(F& f, const char* name) {
    f = reinterpret_cast<F>(dlsym(D.lib, name));
    if (!f) g_err = std::string("missing driver symbol ") + name;
    return f != nullptr;
}

bool load_driver() {
    if (D.lib) return true;
    D.lib = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!D.lib) { g_err = "dlopen libcuda.so.1 failed"; return false; }
    return sym(D.Init, "cuInit") && sym(D.DeviceGet, "cuDeviceGet") &&
           sym(D.DevicePrimaryCtxRetain, "cuDevicePrimaryCtxRetain") &&
           sym(D.DevicePrimaryCtxRelease, "cuDevicePrimaryCtxRelease_v2") &&
           sym(D.CtxSetCurrent, "cuCtxSetCurrent") && sym(D.CtxSynchronize, "cuCtxSynchronize") &&
           sym(D.ModuleLoad, "cuModuleLoad") && sym(D.ModuleUnload, "cuModuleUnload") &&
           sym(D.ModuleGetFunction, "cuModuleGetFunction") && sym(D.ModuleGetGlobal, "cuModuleGetGlobal_v2") &&
           sym(D.MemAlloc, "cuMemAlloc_v2") && sym(D.MemFree, "cuMemFree_v2") && sym(D.MemsetD8, "cuMemsetD8_v2") &&
           sym(D.MemcpyHtoD, "cuMemcpyHtoD_v2") && sym(D.MemcpyDtoH, "cuMemcpyDtoH_v2") &&
           sym(D.MemcpyDtoD, "cuMemcpyDtoD_v2") && sym(D.LaunchKernel, "cuLaunchKernel") &&
           sym(D.GetErrorString, "cuGetErrorString");
}

#define CK(x)                                                             \
    do {                                                                  \
        CUresult r_ = (x);                                                \
        if (r_ != CUDA_SUCCESS) {                                         \
            const char* s_ = nullptr;                                     \
            D.GetErrorString(r_, &s_);                                    \
            g_err = std::string(#x) + ": " + (s_ ? s_ : "?");             \
            return -3;                                                    \
        }                                                                 \
    } while (0)

// ---- mirrors of the reference's device-side structs -----------------------
// struct Parameters, src/global.h:44-108 (REAL = R)
template <typename R>
struct RefParams {
    int nx, ny, nz;
    R Lx, Ly, Lz;
    R Ox, Oy, Oz;
    R dx, dy, dz;
    R dx1, dy1, dz1;
    char bInit[30];
    char uInit[30];
    R ampl;
    R phi1, phi2;
    R L1, L2;
    R ar, az;
    int nBlobs;
    R width;
    R minor_, major_;
    R stretch;
    R bGround;
    R blobXc[10], blobYc[10], blobZc[10], blobZl[10], blobTwist[10], blobScale[10];
    char initDist[30];
    int initDistCode;
    R initShearA, initShearB, initShearK;
    R pert;
    R twist;
    bool fRestart;
    int nCycle;
    R dt0, dtMin, maxError;
    bool zUpdate, inertia, pressure;
    R nu, beta;
    bool jxbAver;
    R jxbAverWeight;
    bool xPeri, yPeri, zPeri;
    bool epsilonProf;
    char jMethod[30];
    char pMethod[30];
    int nTs;
    R dtDump, dtSave;
    bool dumpJ, dumpDetJac, dumpCellVol, dumpConvexity, dumpWedgeMin;
    bool redB2, redB2f, redBMax, redJMax, redJxB_B2Max, redEpsilonStar, redErrB_1ez, redErrXb_XbAn, redConvex,
        redWedgeMin, redU2, redUMax;
};

// struct VarsDev, src/global.h:139-166
struct RefVarsDev {
    CUdeviceptr xb, B0, uu, B, J, gradP, kk, xb_new, maxDelta, xb_tmp, uu_new, uu_tmp, Jmag, JxB_B2, JB_B2, epsStar,
        detJac, cellVol, convexity, wedgeMin, B_1ez2, xb_xbAn, B2_det, U2_det, Umag;
};

template <typename R>
void fill_params(const gm_params* g, RefParams<R>* p) {
    memset(p, 0, sizeof(*p));
    p->nx = g->nx; p->ny = g->ny; p->nz = g->nz;
    p->Lx = (R)g->Lx; p->Ly = (R)g->Ly; p->Lz = (R)g->Lz;
    p->Ox = (R)g->Ox; p->Oy = (R)g->Oy; p->Oz = (R)g->Oz;
    p->dx = (R)g->dx; p->dy = (R)g->dy; p->dz = (R)g->dz;
    p->dx1 = (R)g->dx1; p->dy1 = (R)g->dy1; p->dz1 = (R)g->dz1;
    memcpy(p->bInit, g->bInit, 30); memcpy(p->uInit, g->uInit, 30);
    p->ampl = (R)g->ampl; p->phi1 = (R)g->phi1; p->phi2 = (R)g->phi2;
    p->L1 = (R)g->L1; p->L2 = (R)g->L2; p->ar = (R)g->ar; p->az = (R)g->az;
    p->nBlobs = g->nBlobs;
    p->width = (R)g->width; p->minor_ = (R)g->minor; p->major_ = (R)g->major;
    p->stretch = (R)g->stretch; p->bGround = (R)g->bGround;
    for (int b = 0; b < 10; b++) {
        p->blobXc[b] = (R)g->blobXc[b]; p->blobYc[b] = (R)g->blobYc[b]; p->blobZc[b] = (R)g->blobZc[b];
        p->blobZl[b] = (R)g->blobZl[b]; p->blobTwist[b] = (R)g->blobTwist[b]; p->blobScale[b] = (R)g->blobScale[b];
    }
    memcpy(p->initDist, g->initDist, 30);
    p->initDistCode = g->initDistCode;
    p->initShearA = (R)g->initShearA; p->initShearB = (R)g->initShearB; p->initShearK = (R)g->initShearK;
    p->pert = (R)g->pert; p->twist = (R)g->twist;
    p->fRestart = g->fRestart != 0;
    p->nCycle = g->nCycle;
    p->dt0 = (R)g->dt0; p->dtMin = (R)g->dtMin; p->maxError = (R)g->maxError;
    p->zUpdate = g->zUpdate != 0; p->inertia = g->inertia != 0; p->pressure = g->pressure != 0;
    p->nu = (R)g->nu; p->beta = (R)g->beta;
    p->jxbAver = g->jxbAver != 0; p->jxbAverWeight = (R)g->jxbAverWeight;
    p->xPeri = g->xPeri != 0; p->yPeri = g->yPeri != 0; p->zPeri = g->zPeri != 0;
    p->epsilonProf = g->epsilonProf != 0;
    memcpy(p->jMethod, g->jMethod, 30); memcpy(p->pMethod, g->pMethod, 30);
    p->nTs = g->nTs;
    p->dtDump = (R)g->dtDump; p->dtSave = (R)g->dtSave;
}

struct Dim { unsigned x, y, z; };

// ---- the launcher state ---------------------------------------------------
struct Ref {
    int prec = 0;
    size_t rs = 8;   // sizeof(REAL)
    CUdevice dev = 0;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction fBJ, fBound, fPeri, fJ, fGradP, fKK, fGridPeri, fXNS, fMaxBlock;
    gm_params gp;
    RefVarsDev d;
    CUdeviceptr dmax = 0, dtmp = 0;
    int block[3], grid[3];
    Dim g2XY, g2XZ, g2YZ, g2pXY, g2pXZ, g2pYZ;
    double t = 0, dt = 0, maxDelta = 0;
    int timeIndex = 0, nAttempted = 0;
    size_t NG = 0, N = 0;
    bool open = false;
    bool classic = false;   // jMethod = "Classic": JClassic instead of JStokes
    bool oct = false;       // jMethod = "Stokes4th": JStokes4th (same shared memory as JStokes)
    bool quint = false;     // jMethod = "StokesQuint": JStokesQuint (same shared memory)
    bool tri = false;       // jMethod = "StokesTri": JStokesTri (same shared memory)
};
Ref S;

const char* kname(const char* base, int prec) {
    // Itanium-mangled names of the reference kernels for REAL = double/float.
    static std::string s;
    std::string r = prec == 64 ? "d" : "f";
    std::string b = base;
    if (b == "B_JacB0") s = "_Z7B_JacB07VarsDeviii";
    else if (b == "updateBbound") s = "_Z12updateBbound7VarsDevi";
    else if (b == "setPeriFace") s = "_Z11setPeriFaceP" + r + "i";
    else if (b == "JStokes") s = "_Z7JStokes7VarsDeviii";
    else if (b == "JClassic") s = "_Z8JClassic7VarsDeviii";
    else if (b == "JStokes4th") s = "_Z10JStokes4th7VarsDeviii";
    else if (b == "JStokesQuint") s = "_Z12JStokesQuint7VarsDeviii";
    else if (b == "JStokesTri") s = "_Z10JStokesTri7VarsDeviii";
    else if (b == "gradPClassic") s = "_Z12gradPClassic7VarsDeviii";
    else if (b == "kk") s = "_Z2kk7VarsDeviiii" + r;
    else if (b == "setGridPeriFace") s = "_Z15setGridPeriFaceP" + r + "i";
    else if (b == "xNewStar") s = "_Z8xNewStar7VarsDeviii";
    else if (b == "maxBlock") s = "_Z8maxBlockP" + r + "S_i";
    else if (b == "dirCellVol") s = "_Z10dirCellVolP" + r + "S_iii";
    else if (b == "gridConvexity") s = "_Z13gridConvexityP" + r + "S_iii";
    else if (b == "gridWedgeMin") s = "_Z12gridWedgeMinP" + r + "S_iii";
    else if (b == "JB_B2") s = "_Z5JB_B2P" + r + "S_S_";
    else if (b == "epsilonStar") s = "_Z11epsilonStarP" + r + "S_S_i";
    else if (b == "B_1ez") s = "_Z5B_1ezP" + r + "S_";
    else if (b == "xb_XbAn") s = "_Z7xb_XbAnP" + r + "S_";
    return s.c_str();
}

int get_fn(CUfunction* f, const char* base) {
    CUresult r = D.ModuleGetFunction(f, S.mod, kname(base, S.prec));
    if (r != CUDA_SUCCESS) {
        g_err = std::string("kernel not found in cubin: ") + base + " (" + kname(base, S.prec) + ")";
        return -3;
    }
    return 0;
}

int launch(CUfunction f, Dim g, Dim b, unsigned smem, void** args) {
    CK(D.LaunchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, smem, nullptr, args, nullptr));
    return 0;
}
#define LK(...)                              \
    do {                                     \
        int rc_ = launch(__VA_ARGS__);        \
        if (rc_) return rc_;                 \
    } while (0)
#define SYNC() CK(D.CtxSynchronize())

size_t gbytes() { return 3 * S.NG * S.rs; }

// setBbound, src/boundaries.cu:637-642
int set_b_bound() {
    Dim b16{16, 16, 1};
    int face;
    void* a[2] = {&S.d, &face};
    face = 2; LK(S.fBound, S.g2XY, b16, 0, a); SYNC();
    face = 1; LK(S.fBound, S.g2XZ, b16, 0, a); SYNC();
    face = 0; LK(S.fBound, S.g2YZ, b16, 0, a); SYNC();
    return 0;
}

// setPeri / setGridPeri, src/boundaries.cu:645-658
int set_peri(CUfunction f, CUdeviceptr field) {
    Dim b16{16, 16, 1};
    int face;
    void* a[2] = {&field, &face};
    if (S.gp.zPeri) { face = 2; LK(f, S.g2pXY, b16, 0, a); }
    if (S.gp.yPeri) { face = 1; LK(f, S.g2pXZ, b16, 0, a); }
    if (S.gp.xPeri) { face = 0; LK(f, S.g2pYZ, b16, 0, a); }
    return 0;
}

Dim dgrid() { return Dim{(unsigned)S.grid[0], (unsigned)S.grid[1], (unsigned)S.grid[2]}; }
Dim dblock() { return Dim{(unsigned)S.block[0], (unsigned)S.block[1], (unsigned)S.block[2]}; }

// B_JacB0 + setBbound + setPeri(B) + current, src/main.cu:262-272
int fields() {
    int b0 = S.block[0], b1 = S.block[1], b2 = S.block[2];
    int dX = b0 + 2, dY = b1 + 2, dZ = b2 + 2;
    void* a[4] = {&S.d, &dX, &dY, &dZ};
    LK(S.fBJ, dgrid(), dblock(), (unsigned)(3 * dX * dY * dZ * 3 * S.rs), a);
    SYNC();
    int rc = set_b_bound();
    if (rc) return rc;
    rc = set_peri(S.fPeri, S.d.B);
    if (rc) return rc;
    SYNC();
    // current(), src/current.cu:1685-1720: dynamic shared memory per method
    const unsigned jsm = S.classic ? (unsigned)(dX * dY * dZ * (3 * 2 + 1) * S.rs)
                                   : (unsigned)((3 * dX * dY * dZ * 2 + 3 * b0 * b1 * b2) * S.rs);
    LK(S.fJ, dgrid(), dblock(), jsm, a);
    SYNC();
    return 0;
}

int stage(int n) {
    int b0 = S.block[0], b1 = S.block[1], b2 = S.block[2];
    int dX = b0 + 2, dY = b1 + 2, dZ = b2 + 2;
    int rc = fields();
    if (rc) return rc;
    if (S.gp.pressure) {
        void* a[4] = {&S.d, &dX, &dY, &dZ};
        LK(S.fGradP, dgrid(), dblock(), (unsigned)(dX * dY * dZ * 3 * S.rs), a);
    }
    SYNC();
    unsigned smem = (unsigned)(b0 * b1 * b2 * (3 * (9 + 7 * S.gp.inertia + S.gp.pressure) + S.gp.inertia) * S.rs);
    if (S.prec == 64) {
        double dt = S.dt;
        void* a[6] = {&S.d, &dX, &dY, &dZ, &n, &dt};
        LK(S.fKK, dgrid(), dblock(), smem, a);
    } else {
        float dt = (float)S.dt;
        void* a[6] = {&S.d, &dX, &dY, &dZ, &n, &dt};
        LK(S.fKK, dgrid(), dblock(), smem, a);
    }
    SYNC();
    rc = set_peri(S.fGridPeri, S.d.xb);
    if (rc) return rc;
    rc = set_peri(S.fGridPeri, S.d.xb_tmp);
    if (rc) return rc;
    SYNC();
    CK(D.MemcpyDtoD(S.d.xb, S.d.xb_tmp, gbytes()));
    if (S.gp.inertia) CK(D.MemcpyDtoD(S.d.uu, S.d.uu_tmp, 3 * S.N * S.rs));   // main.cu:296-305
    SYNC();
    return 0;
}

// findDevMax, src/maths.cu:101-130
int find_dev_max(CUdeviceptr var, int size, double* out) {
    CK(D.MemcpyDtoD(S.dmax, var, (size_t)size * S.rs));
    Dim b32{32, 1, 1};
    while (size > 1) {
        unsigned nb = (unsigned)ceil(size / 64.);
        void* a[3] = {&S.dmax, &S.dtmp, &size};
        LK(S.fMaxBlock, Dim{nb, 1, 1}, b32, 0, a);
        SYNC();
        CK(D.MemcpyDtoD(S.dmax, S.dtmp, nb * S.rs));
        SYNC();
        size = (int)nb;
    }
    if (S.prec == 64) {
        double v;
        CK(D.MemcpyDtoH(&v, S.dmax, sizeof v));
        *out = v;
    } else {
        float v;
        CK(D.MemcpyDtoH(&v, S.dmax, sizeof v));
        *out = v;
    }
    return 0;
}

int combine() {
    int b0 = S.block[0], b1 = S.block[1], b2 = S.block[2];
    int dX = b0 + 2, dY = b1 + 2, dZ = b2 + 2;
    void* a[4] = {&S.d, &dX, &dY, &dZ};
    LK(S.fXNS, dgrid(), dblock(), (unsigned)(3 * (10 + 9 * S.gp.inertia) * b0 * b1 * b2 * S.rs), a);
    SYNC();
    int rc = set_peri(S.fGridPeri, S.d.xb_new);
    if (rc) return rc;
    SYNC();
    return find_dev_max(S.d.maxDelta, S.grid[0] * S.grid[1] * S.grid[2], &S.maxDelta);
}

double to_real(double v) { return S.prec == 64 ? v : (double)(float)v; }

// the loop body of src/main.cu:259-384 without diagnostics and dumps
int step(int nCycle, int* accepted) {
    if (!(S.timeIndex < nCycle && S.dt > S.gp.dtMin)) { *accepted = -1; return 0; }
    for (int n = 0; n < 6; n++) {
        int rc = stage(n);
        if (rc) return rc;
    }
    int rc = combine();
    if (rc) return rc;
    S.nAttempted++;
    double ex = S.prec == 64 ? 0.2 : (double)0.2f;
    if (S.maxDelta < S.gp.maxError) {
        S.t = to_real(S.t + S.dt);
        CK(D.MemcpyDtoD(S.d.xb, S.d.xb_new, gbytes()));
        if (S.gp.inertia) CK(D.MemcpyDtoD(S.d.uu, S.d.uu_new, 3 * S.N * S.rs));   // main.cu:331-339
        SYNC();
        rc = fields();
        if (rc) return rc;
        if (S.maxDelta > 0) S.dt = to_real(S.dt * pow(0.9 * S.gp.maxError / S.maxDelta, ex));
        S.timeIndex++;
        *accepted = 1;
    } else {
        if (S.maxDelta > 0) S.dt = to_real(S.dt * pow(0.9 * S.gp.maxError / S.maxDelta, ex));
        *accepted = 0;
    }
    return 0;
}

int alloc(CUdeviceptr* p, size_t bytes) {
    CK(D.MemAlloc(p, bytes));
    CK(D.MemsetD8(*p, 0, bytes));
    return 0;
}

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

void ref_close(void) {
    if (!S.open) return;
    CUdeviceptr* ps = reinterpret_cast<CUdeviceptr*>(&S.d);
    for (size_t i = 0; i < sizeof(S.d) / sizeof(CUdeviceptr); i++)
        if (ps[i]) D.MemFree(ps[i]);
    if (S.dmax) D.MemFree(S.dmax);
    if (S.dtmp) D.MemFree(S.dtmp);
    if (S.mod) D.ModuleUnload(S.mod);
    D.DevicePrimaryCtxRelease(S.dev);
    S = Ref();
}

// Load the cubin and set up a run of the given parameters and initial state
// (host arrays in the reference layout).  Mirrors src/memory.cu:10-72 and
// src/main.cu:128-256 (device buffers are zero-filled here).
int ref_open(const char* cubin, const gm_params* g, const void* B0, const void* xb, double t, double dt) {
    if (!load_driver()) return -3;
    ref_close();
    S.classic = strncmp(g->jMethod, "Classic ", 8) == 0;
    S.oct = strncmp(g->jMethod, "Stokes4th ", 10) == 0;
    S.quint = strncmp(g->jMethod, "StokesQuint ", 12) == 0;
    S.tri = strncmp(g->jMethod, "StokesTri ", 10) == 0;
    if (strncmp(g->jMethod, "Stokes ", 7) != 0 && !S.classic && !S.oct && !S.quint && !S.tri) {
        g_err = "only jMethod = Stokes, Stokes4th, StokesQuint, StokesTri or Classic";
        return -1;
    }
    S.prec = g->precision;
    S.rs = S.prec == 64 ? 8 : 4;
    S.gp = *g;
    CK(D.Init(0));
    CK(D.DeviceGet(&S.dev, 0));
    CK(D.DevicePrimaryCtxRetain(&S.ctx, S.dev));
    CK(D.CtxSetCurrent(S.ctx));
    S.open = true;
    CK(D.ModuleLoad(&S.mod, cubin));
    int rc = 0;
    if ((rc = get_fn(&S.fBJ, "B_JacB0")) || (rc = get_fn(&S.fBound, "updateBbound")) ||
        (rc = get_fn(&S.fPeri, "setPeriFace")) || (rc = get_fn(&S.fJ, S.classic ? "JClassic" : (S.oct ? "JStokes4th" : (S.quint ? "JStokesQuint" : (S.tri ? "JStokesTri" : "JStokes"))))) ||
        (rc = get_fn(&S.fGradP, "gradPClassic")) || (rc = get_fn(&S.fKK, "kk")) ||
        (rc = get_fn(&S.fGridPeri, "setGridPeriFace")) || (rc = get_fn(&S.fXNS, "xNewStar")) ||
        (rc = get_fn(&S.fMaxBlock, "maxBlock")))
        return rc;
    // constant memory: parameters and the Cash-Karp tableau (main.cu:227-256,
    // rungeKutta.cu:10-25)
    CUdeviceptr sp;
    size_t ssz;
    CK(D.ModuleGetGlobal(&sp, &ssz, S.mod, "dev_params"));
    if (S.prec == 64) {
        RefParams<double> rp;
        if (ssz != sizeof rp) { g_err = "struct Parameters size mismatch (double)"; return -1; }
        fill_params(g, &rp);
        CK(D.MemcpyHtoD(sp, &rp, sizeof rp));
    } else {
        RefParams<float> rp;
        if (ssz != sizeof rp) { g_err = "struct Parameters size mismatch (float)"; return -1; }
        fill_params(g, &rp);
        CK(D.MemcpyHtoD(sp, &rp, sizeof rp));
    }
    {
        static const double a[6] = {0, 0.2, 0.3, 0.6, 1, 0.875};
        static const double b[7][6] = {
            {0, 0, 0, 0, 0, 0},
            {0.2, 0, 0, 0, 0, 0},
            {3 / 40., 9 / 40., 0, 0, 0, 0},
            {0.3, -0.9, 1.2, 0, 0, 0},
            {-11 / 54., 2.5, -70 / 27., 35 / 27., 0, 0},
            {1631 / 55296., 175 / 512., 575 / 13824., 44275 / 110592., 253 / 4096., 0},
            {0, 0, 0, 0, 0, 0}};
        static const double c[6] = {37 / 378., 0, 250 / 621., 125 / 594., 0, 512 / 1771.};
        static const double cs[6] = {2825 / 27648., 0, 18575 / 48384., 13525 / 55296., 277 / 14336., 0.25};
        const char* names[4] = {"a_i", "b_ij", "c_i", "cs_i"};
        const double* src[4] = {a, &b[0][0], c, cs};
        int cnt[4] = {6, 42, 6, 6};
        for (int q = 0; q < 4; q++) {
            CK(D.ModuleGetGlobal(&sp, &ssz, S.mod, names[q]));
            if (S.prec == 64) {
                CK(D.MemcpyHtoD(sp, src[q], cnt[q] * sizeof(double)));
            } else {
                float f[42];
                for (int i = 0; i < cnt[q]; i++) f[i] = (float)src[q][i];
                CK(D.MemcpyHtoD(sp, f, cnt[q] * sizeof(float)));
            }
        }
    }
    // block and grid shapes, src/main.cu:130-157
    int E = S.prec == 32 ? 1 : 0;
    S.block[0] = 5 + E; S.block[1] = 6 + E; S.block[2] = 6 + E;
    if (g->inertia) { S.block[1] = 5 + E; S.block[2] = 4 + E; }
    S.grid[0] = (g->nx - 1) / S.block[0] + 1;
    S.grid[1] = (g->ny - 1) / S.block[1] + 1;
    S.grid[2] = (g->nz - 1) / S.block[2] + 1;
    S.g2pXY = Dim{(unsigned)((g->nx + 1) / 16 + 1), (unsigned)((g->ny + 1) / 16 + 1), 1};
    S.g2pXZ = Dim{(unsigned)((g->nx + 1) / 16 + 1), (unsigned)((g->nz + 1) / 16 + 1), 1};
    S.g2pYZ = Dim{(unsigned)((g->ny + 1) / 16 + 1), (unsigned)((g->nz + 1) / 16 + 1), 1};
    S.g2XY = Dim{(unsigned)((g->nx - 1) / 16 + 1), (unsigned)((g->ny - 1) / 16 + 1), 1};
    S.g2XZ = Dim{(unsigned)((g->nx - 1) / 16 + 1), (unsigned)((g->nz - 1) / 16 + 1), 1};
    S.g2YZ = Dim{(unsigned)((g->ny - 1) / 16 + 1), (unsigned)((g->nz - 1) / 16 + 1), 1};
    // memory, src/memory.cu:38-72
    S.NG = (size_t)(g->nx + 2) * (g->ny + 2) * (g->nz + 2);
    S.N = (size_t)g->nx * g->ny * g->nz;
    size_t v = 3 * S.NG * S.rs, vi = 3 * S.N * S.rs;
    size_t nblk = (size_t)S.grid[0] * S.grid[1] * S.grid[2];
    if ((rc = alloc(&S.d.B0, v)) || (rc = alloc(&S.d.B, v)) || (rc = alloc(&S.d.xb, v)) || (rc = alloc(&S.d.J, vi)) ||
        (rc = alloc(&S.d.xb_new, v)) || (rc = alloc(&S.d.xb_tmp, v)) || (rc = alloc(&S.d.kk, 6 * vi)) ||
        (rc = alloc(&S.d.gradP, vi)) || (rc = alloc(&S.d.maxDelta, nblk * S.rs)) ||
        (rc = alloc(&S.d.detJac, S.NG * S.rs)) || (rc = alloc(&S.dmax, nblk * S.rs)) ||
        (rc = alloc(&S.dtmp, (nblk / 64 + 2) * S.rs)))
        return rc;
    if (g->inertia) {
        // kk holds 6 variables per point; uu starts at zero (uInit = "nil")
        if ((rc = alloc(&S.d.uu, vi)) || (rc = alloc(&S.d.uu_tmp, vi)) || (rc = alloc(&S.d.uu_new, vi))) return rc;
        D.MemFree(S.d.kk);
        S.d.kk = 0;
        if ((rc = alloc(&S.d.kk, 12 * vi))) return rc;
    }
    // initial copies, src/main.cu:181-215
    CK(D.MemcpyHtoD(S.d.B0, B0, v));
    CK(D.MemcpyHtoD(S.d.xb, xb, v));
    CK(D.MemcpyDtoD(S.d.B, S.d.B0, v));
    CK(D.MemcpyDtoD(S.d.xb_tmp, S.d.xb, v));
    CK(D.MemcpyDtoD(S.d.xb_new, S.d.xb, v));
    SYNC();
    S.t = to_real(t);
    S.dt = to_real(dt);
    S.timeIndex = 0;
    S.nAttempted = 0;
    return 0;
}

int ref_stage(int n) { return stage(n); }
int ref_combine(double* maxDelta) {
    int rc = combine();
    if (maxDelta) *maxDelta = S.maxDelta;
    return rc;
}
int ref_refresh(void) { return fields(); }

int ref_step(int nCycle, int* accepted) { return step(nCycle, accepted); }

// Attempted steps until nCycle accepted or dt <= dtMin or maxAttempts;
// log[3a..3a+2] = (maxDelta, dt after the update, accepted).
int ref_run(int nCycle, int maxAttempts, double* log, int* nDone) {
    int a = 0;
    while (a < maxAttempts) {
        int acc = 0;
        int rc = step(nCycle, &acc);
        if (rc) return rc;
        if (acc < 0) break;
        if (log) {
            log[3 * a] = S.maxDelta;
            log[3 * a + 1] = S.dt;
            log[3 * a + 2] = acc;
        }
        a++;
    }
    if (nDone) *nDone = a;
    return 0;
}

// Wall time of `nAttempts` attempted steps of the reference (host loop with
// its device synchronisations), for the reference-build baseline.
int ref_time_steps(int nAttempts, double* seconds, int* nDone) {
    SYNC();
    auto t0 = std::chrono::steady_clock::now();
    int a = 0;
    for (; a < nAttempts; a++) {
        int acc;
        int rc = step(1 << 30, &acc);
        if (rc) return rc;
        if (acc < 0) break;
    }
    SYNC();
    auto t1 = std::chrono::steady_clock::now();
    *seconds = std::chrono::duration<double>(t1 - t0).count();
    if (nDone) *nDone = a;
    return 0;
}

int ref_get(void* xb, void* B, void* J, void* detJac) {
    SYNC();
    if (xb) CK(D.MemcpyDtoH(xb, S.d.xb, 3 * S.NG * S.rs));
    if (B) CK(D.MemcpyDtoH(B, S.d.B, 3 * S.NG * S.rs));
    if (J) CK(D.MemcpyDtoH(J, S.d.J, 3 * S.N * S.rs));
    if (detJac) CK(D.MemcpyDtoH(detJac, S.d.detJac, S.NG * S.rs));
    return 0;
}

int ref_get_k(int m, void* k) {
    SYNC();
    const size_t nv = S.gp.inertia ? 6 : 3;
    CK(D.MemcpyDtoH(k, S.d.kk + (CUdeviceptr)(nv * S.N * S.rs * (size_t)m), nv * S.N * S.rs));
    return 0;
}

// velocity (inertia): 0 the current uu, 1 uu_new of the last combine
int ref_get_u(int which, void* u) {
    SYNC();
    if (!S.gp.inertia) { g_err = "no velocity without inertia"; return -1; }
    CK(D.MemcpyDtoH(u, which ? S.d.uu_new : S.d.uu, 3 * S.N * S.rs));
    return 0;
}

int ref_get_xnew(void* x) {
    SYNC();
    CK(D.MemcpyDtoH(x, S.d.xb_new, 3 * S.NG * S.rs));
    return 0;
}

// The per-point grid fields of prepareDump (src/diagnostics.cu:154-190):
// dirCellVol, gridConvexity and gridWedgeMin on the current grid, with the
// run's block and grid shapes and dynamic shared-memory sizes, copied to the
// host arrays (inner layout, REAL; any pointer may be NULL).
int ref_grid_fields(void* cellVol, void* convexity, void* wedgeMin) {
    const int b0 = S.block[0], b1 = S.block[1], b2 = S.block[2];
    const size_t vi = S.N * S.rs;
    CUdeviceptr out = 0;
    CK(D.MemAlloc(&out, vi));
    int rc = 0;
    struct Job { const char* name; void* host; int pad; unsigned smem; };
    const Job jobs[3] = {
        {"dirCellVol", cellVol, 1, (unsigned)((3 * (b0 + 1) * (b1 + 1) * (b2 + 1) + b0 * b1 * b2) * S.rs)},
        {"gridConvexity", convexity, 2, (unsigned)((3 * (b0 + 2) * (b1 + 2) * (b2 + 2) + b0 * b1 * b2) * S.rs)},
        {"gridWedgeMin", wedgeMin, 2, (unsigned)(3 * (b0 + 2) * (b1 + 2) * (b2 + 2) * S.rs)}};
    for (const Job& j : jobs) {
        if (!j.host) continue;
        CUfunction f;
        if ((rc = get_fn(&f, j.name))) break;
        int dX = b0 + j.pad, dY = b1 + j.pad, dZ = b2 + j.pad;
        CUdeviceptr xb = S.d.xb;
        void* a[5] = {&xb, &out, &dX, &dY, &dZ};
        if ((rc = launch(f, dgrid(), dblock(), j.smem, a))) break;
        if (D.CtxSynchronize() != CUDA_SUCCESS || D.MemcpyDtoH(j.host, out, vi) != CUDA_SUCCESS) {
            g_err = std::string("ref_grid_fields: ") + j.name;
            rc = -3;
            break;
        }
    }
    D.MemFree(out);
    return rc;
}

// eps* as src/diagnostics.cu:32-47 computes it: JB_B2, then epsilonStar
// over the nz x nz pairs, then findDevMax.  The reference's kernel covers
// every pair only for nz <= 256 or a multiple of 256 (its block size), so
// other nz are refused.
int ref_eps_star(double* out) {
    const int nz = S.gp.nz;
    if (!(nz <= 256 || nz % 256 == 0)) { g_err = "ref_eps_star: nz must be <= 256 or a multiple of 256"; return -1; }
    CUfunction fjb, feps;
    int rc = 0;
    if ((rc = get_fn(&fjb, "JB_B2")) || (rc = get_fn(&feps, "epsilonStar"))) return rc;
    CUdeviceptr jb = 0, eps = 0;
    CK(D.MemAlloc(&jb, (size_t)nz * S.rs));
    if (D.MemAlloc(&eps, (size_t)nz * nz * S.rs) != CUDA_SUCCESS) { D.MemFree(jb); g_err = "ref_eps_star: alloc"; return -3; }
    CUdeviceptr B = S.d.B, J = S.d.J, xb = S.d.xb;
    int dimZ = 256;
    void* a1[3] = {&B, &J, &jb};
    void* a2[4] = {&xb, &jb, &eps, &dimZ};
    const unsigned nb = (unsigned)((nz - 1) / 256 + 1);
    rc = launch(fjb, Dim{nb, 1, 1}, Dim{256, 1, 1}, 0, a1);
    if (!rc && D.CtxSynchronize() != CUDA_SUCCESS) { g_err = "ref_eps_star: JB_B2"; rc = -3; }
    if (!rc) rc = launch(feps, Dim{nb, 1, 1}, Dim{256, 1, 1}, (unsigned)(512 * 2 * S.rs), a2);
    if (!rc && D.CtxSynchronize() != CUDA_SUCCESS) { g_err = "ref_eps_star: epsilonStar"; rc = -3; }
    // findDevMax uses the launcher's own scratch, sized for the step's block
    // maxima: reduce here when the pair count fits it, else on the host
    if (!rc) {
        const size_t cnt = (size_t)nz * nz;
        const size_t nblk = (size_t)S.grid[0] * S.grid[1] * S.grid[2];
        if (cnt <= nblk) {
            rc = find_dev_max(eps, (int)cnt, out);
        } else {
            std::vector<double> h(cnt);
            if (S.prec == 64) {
                if (D.MemcpyDtoH(h.data(), eps, cnt * 8) != CUDA_SUCCESS) rc = -3;
            } else {
                std::vector<float> hf(cnt);
                if (D.MemcpyDtoH(hf.data(), eps, cnt * 4) != CUDA_SUCCESS) rc = -3;
                for (size_t q = 0; q < cnt; q++) h[q] = hf[q];
            }
            double m = 0;   // every value is >= 0; NaN never wins (maxBlock's compare)
            for (double v : h)
                if (v > m) m = v;
            *out = m;
            if (rc) g_err = "ref_eps_star: copy";
        }
    }
    D.MemFree(jb);
    D.MemFree(eps);
    return rc;
}

// errB_1ez and errXb_XbAn as src/diagnostics.cu:51-71 form them: the
// kernels' per-block partial sums (B_1ez, xb_XbAn, 256 threads), summed on
// the host in double, then sqrt(sum) / sqrt(N).
int ref_errors(double* errB, double* errXb) {
    CUfunction fb, fx;
    int rc = 0;
    if ((rc = get_fn(&fb, "B_1ez")) || (rc = get_fn(&fx, "xb_XbAn"))) return rc;
    const unsigned nb = (unsigned)((S.N - 1) / 256 + 1);
    CUdeviceptr part = 0;
    CK(D.MemAlloc(&part, (size_t)nb * S.rs));
    double* outs[2] = {errB, errXb};
    CUfunction fs[2] = {fb, fx};
    CUdeviceptr src[2] = {S.d.B, S.d.xb};
    for (int q = 0; q < 2 && !rc; q++) {
        void* a[2] = {&src[q], &part};
        rc = launch(fs[q], Dim{nb, 1, 1}, Dim{256, 1, 1}, 0, a);
        if (rc) break;
        if (D.CtxSynchronize() != CUDA_SUCCESS) { g_err = "ref_errors: kernel"; rc = -3; break; }
        double sum = 0;
        if (S.prec == 64) {
            std::vector<double> h(nb);
            if (D.MemcpyDtoH(h.data(), part, (size_t)nb * 8) != CUDA_SUCCESS) { rc = -3; break; }
            for (double v : h) sum += v;
        } else {
            std::vector<float> h(nb);
            if (D.MemcpyDtoH(h.data(), part, (size_t)nb * 4) != CUDA_SUCCESS) { rc = -3; break; }
            for (float v : h) sum += v;
        }
        *outs[q] = sqrt(sum) / sqrt((double)S.N);
    }
    D.MemFree(part);
    return rc;
}

void ref_scalars(double* out) {
    out[0] = S.t; out[1] = S.dt; out[2] = S.maxDelta; out[3] = S.timeIndex; out[4] = S.nAttempted;
}

}  // extern "C"
