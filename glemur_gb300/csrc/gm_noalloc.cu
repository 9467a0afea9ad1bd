// gm_noalloc.cu -- force-free residual and field reductions without any
// device allocation.
//
// Some callers cannot allocate device memory at the point where they want the
// relaxation diagnostics: an application whose GPU memory is owned by its own
// pool allocator (a framework that reserved the device's memory up front, so a
// cudaMalloc from a library fails or escapes the pool's accounting), a
// stream-ordered pipeline that must not stall (cudaFree, and cudaMalloc in
// places, synchronise the device), or a service with a fixed memory budget
// that allocates nothing after start-up.  gm_reduce_noalloc gives them the
// reductions of gm_refresh from B, J and detJac arrays they already hold, with
// the per-plane partial sums kept in a fixed file-scope device array instead
// of handle-owned scratch.
#include <cuda_runtime.h>

#include <float.h>
#include <math.h>

#include <mutex>
#include <string>

#include "glemur.h"
#include "gm_internal.h"

namespace {

constexpr int kFields = 16;   // per-plane partial: 7 sums + 4 maxima/minima, padded
enum { S_CROSS = 0, S_JB, S_PW, S_B2W, S_E1, M_JXBB2, M_B, M_J, N_DET };

// Scratch: one partial per z-plane.  Every GPU that loads this library holds
// it (GM_NOALLOC_MAX_PLANES * 16 doubles = 512 KiB) until the process exits.
__device__ __align__(256) double g_plane_partials[GM_NOALLOC_MAX_PLANES * kFields];

constexpr int kMaxDevices = 64;
// device address of g_plane_partials per device, set by the first successful
// lookup (a failed lookup is not cached: the next call tries again)
std::mutex g_setup_mutex;
double* g_scratch[kMaxDevices] = {nullptr};

// The device address of the scratch array on device `dev` (current).
cudaError_t scratch_address(int dev, double** out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch[dev]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_plane_partials);
        if (e != cudaSuccess) return e;
        g_scratch[dev] = static_cast<double*>(ptr);
    }
    *out = g_scratch[dev];
    return cudaSuccess;
}

// One CTA per z-plane: inner points of plane k and, for line-tied faces, the
// ghost-plane detJac values next to them (the minDetJac of gm_refresh).
template <typename T>
__global__ void __launch_bounds__(256) k_plane_partials(const T* __restrict__ B, const T* __restrict__ J,
                                                         const T* __restrict__ D, int nx, int ny, int nz, int xPeri,
                                                         int yPeri, int zPeri, double* __restrict__ part) {
    const int k = blockIdx.x;
    double s[5] = {0, 0, 0, 0, 0};
    double mjxb = 0, mb = 0, mj = 0, mdet = DBL_MAX;
    const long long gx = nx + 2, gxy = (long long)(nx + 2) * (ny + 2);
    for (int q = threadIdx.x; q < nx * ny; q += blockDim.x) {
        const int i = q % nx, j = q / nx;
        const long long g = (i + 1) + gx * (j + 1) + gxy * (k + 1);
        const long long lin = i + (long long)nx * (j + (long long)ny * k);
        const T b0 = B[3 * g], b1 = B[3 * g + 1], b2 = B[3 * g + 2];
        const T j0 = J[3 * lin], j1 = J[3 * lin + 1], j2 = J[3 * lin + 2];
        const T Dv = D[g];
        // |JxB|/B^2 in the run precision (src/maths.cu:168-200)
        const T c0 = j1 * b2 - j2 * b1, c1 = j2 * b0 - j0 * b2, c2 = j0 * b1 - j1 * b0;
        const T bb = b0 * b0 + b1 * b1 + b2 * b2;
        const T q1 = sqrt(c0 * c0 + c1 * c1 + c2 * c2) / bb;
        const double bx = b0, by = b1, bz = b2, jx = j0, jy = j1, jz = j2;
        const double bn = sqrt(bx * bx + by * by + bz * bz), jn = sqrt(jx * jx + jy * jy + jz * jz);
        const double cx = jy * bz - jz * by, cy = jz * bx - jx * bz, cz = jx * by - jy * bx;
        const double cn = sqrt(cx * cx + cy * cy + cz * cz);
        s[0] += cn;
        s[1] += jn * bn;
        if (jn * bn > 0) s[2] += cn / (jn * bn);
        const int bound = (i == 0) + (j == 0) + (k == 0) + (i == nx - 1) + (j == ny - 1) + (k == nz - 1);
        s[3] += (double)bb * (double)Dv / (double)(1 << bound);
        s[4] += bx * bx + by * by + (bz - 1.0) * (bz - 1.0);
        mjxb = fmax(mjxb, (double)q1);
        mb = fmax(mb, bn);
        mj = fmax(mj, jn);
        mdet = fmin(mdet, (double)Dv);
        // ghost planes of line-tied faces adjacent to this point
        if (!xPeri && i == 0) mdet = fmin(mdet, (double)D[0 + gx * (j + 1) + gxy * (k + 1)]);
        if (!xPeri && i == nx - 1) mdet = fmin(mdet, (double)D[(nx + 1) + gx * (j + 1) + gxy * (k + 1)]);
        if (!yPeri && j == 0) mdet = fmin(mdet, (double)D[(i + 1) + gxy * (k + 1)]);
        if (!yPeri && j == ny - 1) mdet = fmin(mdet, (double)D[(i + 1) + gx * (ny + 1) + gxy * (k + 1)]);
        if (!zPeri && k == 0) mdet = fmin(mdet, (double)D[(i + 1) + gx * (j + 1)]);
        if (!zPeri && k == nz - 1) mdet = fmin(mdet, (double)D[(i + 1) + gx * (j + 1) + gxy * (nz + 1)]);
    }
    // fixed-order CTA reduction
    __shared__ double red[9][256];
    const int t = threadIdx.x;
    red[0][t] = s[0]; red[1][t] = s[1]; red[2][t] = s[2]; red[3][t] = s[3]; red[4][t] = s[4];
    red[5][t] = mjxb; red[6][t] = mb; red[7][t] = mj; red[8][t] = mdet;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (t < w) {
            for (int f = 0; f < 5; f++) red[f][t] += red[f][t + w];
            for (int f = 5; f < 8; f++) red[f][t] = fmax(red[f][t], red[f][t + w]);
            red[8][t] = fmin(red[8][t], red[8][t + w]);
        }
        __syncthreads();
    }
    if (t < 9) part[(long long)k * kFields + t] = red[t][0];
}

// Fixed-order reduction of the nz plane partials into a gm_reduction.
__global__ void k_plane_final(const double* __restrict__ part, int nz, double N, double dxdydz,
                              gm_reduction* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double s[5] = {0, 0, 0, 0, 0}, m[3] = {0, 0, 0}, mdet = DBL_MAX;
    for (int k = 0; k < nz; k++) {
        const double* p = part + (long long)k * kFields;
        for (int f = 0; f < 5; f++) s[f] += p[f];
        for (int f = 0; f < 3; f++) m[f] = fmax(m[f], p[5 + f]);
        mdet = fmin(mdet, p[N_DET]);
    }
    out->B2 = s[S_B2W] * dxdydz;
    out->BMax = m[1];
    out->JMax = m[2];
    out->JxB_B2Max = m[0];
    out->residual = s[S_JB] > 0 ? s[S_CROSS] / s[S_JB] : 0.0;
    out->residualPw = s[S_PW] / N;
    out->minDetJac = mdet;
    out->wedgeMin = nan("");      // needs the grid positions
    out->convex = nan("");
    out->errB_1ez = sqrt(s[S_E1]) / sqrt(N);
    out->errXb_XbAn = nan("");
    out->U2 = nan("");            // needs the velocity
    out->UMax = nan("");
}

}  // namespace

extern "C" int gm_reduce_noalloc(const gm_params* p, const void* B, const void* J, const void* detJac,
                                 gm_reduction* out, void* stream) {
    if (!p || !B || !J || !detJac || !out) return gm::fail(GM_EPARAM, "gm_reduce_noalloc: null argument");
    if (p->precision != 32 && p->precision != 64) return gm::fail(GM_EPARAM, "gm_reduce_noalloc: precision must be 32 or 64");
    if (p->nx < 1 || p->ny < 1 || p->nz < 1) return gm::fail(GM_EPARAM, "gm_reduce_noalloc: empty grid");
    if (p->nz > GM_NOALLOC_MAX_PLANES)
        return gm::fail(GM_EPARAM, "gm_reduce_noalloc: nz = " + std::to_string(p->nz) + " exceeds the scratch limit of " +
                                       std::to_string(GM_NOALLOC_MAX_PLANES) + " planes");
    if ((long long)p->nx * p->ny > (1ll << 30)) return gm::fail(GM_EPARAM, "gm_reduce_noalloc: plane too large");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return gm::fail(GM_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return gm::fail(GM_EPARAM, "gm_reduce_noalloc: device index out of range");
    // An error the caller left pending would otherwise be read back below as
    // this call's launch failure: report it, and leave it pending.
    e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return gm::fail(GM_ECUDA, std::string("gm_reduce_noalloc: a CUDA error was pending before the call: ") +
                                      cudaGetErrorString(e));
    // First call on a device: resolve the device address of the scratch array
    // with that device current (retried on the next call if it fails).
    double* scratch = nullptr;
    e = scratch_address(dev, &scratch);
    if (e != cudaSuccess) return gm::fail(GM_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const double N = (double)p->nx * p->ny * p->nz;
    if (p->precision == 32)
        k_plane_partials<float><<<p->nz, 256, 0, s>>>((const float*)B, (const float*)J, (const float*)detJac, p->nx,
                                                       p->ny, p->nz, p->xPeri, p->yPeri, p->zPeri, scratch);
    else
        k_plane_partials<double><<<p->nz, 256, 0, s>>>((const double*)B, (const double*)J, (const double*)detJac,
                                                        p->nx, p->ny, p->nz, p->xPeri, p->yPeri, p->zPeri,
                                                        scratch);
    k_plane_final<<<1, 32, 0, s>>>(scratch, p->nz, N, p->dx * p->dy * p->dz, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return gm::fail(GM_ECUDA, std::string("gm_reduce_noalloc launch: ") + cudaGetErrorString(e));
    return GM_OK;
}
