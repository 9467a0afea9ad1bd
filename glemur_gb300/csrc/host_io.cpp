// host_io.cpp -- the run-directory files of the reference (src/io.cu): cuda.info,
// data/B0.vtk, data/dump<n>.vtk / data/save.vtk (legacy VTK, big-endian binary
// payloads) and the data/time_series.dat lines, byte for byte, plus the
// restart reader.  Host code only; REAL is float or double by p->precision.
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "glemur.h"
#include "gm_internal.h"

namespace {

// Big-endian encoding of REAL / int values (floatSwap / intSwap, io.cu:86-138).
void put_be(std::vector<unsigned char>& out, const void* v, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(v);
    const uint32_t one = 1;
    const bool little = *reinterpret_cast<const unsigned char*>(&one) == 1;
    for (size_t q = 0; q < n; q++) out.push_back(little ? b[n - 1 - q] : b[q]);
}

template <typename T>
void get_be(const unsigned char* b, T* v) {
    unsigned char tmp[sizeof(T)];
    const uint32_t one = 1;
    const bool little = *reinterpret_cast<const unsigned char*>(&one) == 1;
    for (size_t q = 0; q < sizeof(T); q++) tmp[q] = little ? b[sizeof(T) - 1 - q] : b[q];
    memcpy(v, tmp, sizeof(T));
}

template <typename T>
struct Writer {
    FILE* f;
    std::vector<unsigned char> buf;
    bool ok = true;
    explicit Writer(FILE* fd) : f(fd) { buf.reserve(1 << 20); }
    void text(const char* fmt, ...) __attribute__((format(printf, 2, 3)));
    void real(double v) {
        const T x = (T)v;
        put_be(buf, &x, sizeof(T));
        if (buf.size() >= (1u << 20)) flush();
    }
    void i32(int v) {
        const int32_t x = v;
        put_be(buf, &x, 4);
    }
    void flush() {
        if (!buf.empty() && fwrite(buf.data(), 1, buf.size(), f) != buf.size()) ok = false;
        buf.clear();
    }
};

template <typename T>
void Writer<T>::text(const char* fmt, ...) {
    flush();
    va_list ap;
    va_start(ap, fmt);
    if (vfprintf(f, fmt, ap) < 0) ok = false;
    va_end(ap);
}

template <typename T>
const char* real_str() {
    return sizeof(T) == 4 ? "float" : "double";
}

// REAL arithmetic of the reference on parameters held as widened doubles.
template <typename T>
inline T R(double v) {
    return (T)v;
}

template <typename T>
int write_b0(const gm_params* p, const char* path, const T* B0) {
    FILE* f = fopen(path, "wb");
    if (!f) return gm::fail(GM_EIO, std::string("error: could not open file '") + path + "'");
    Writer<T> w(f);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    w.text("# vtk DataFile Version 2.0\n");
    w.text("GLEMuR B0 dump\n");
    w.text("BINARY\n");
    w.text("DATASET STRUCTURED_POINTS\n");
    w.text("DIMENSIONS %9i %9i %9i\n", nx + 2, ny + 2, nz + 2);
    w.text("ORIGIN %8.12f %8.12f %8.12f\n", (double)(T)(R<T>(p->Ox) - R<T>(p->dx)),
           (double)(T)(R<T>(p->Oy) - R<T>(p->dy)), (double)(T)(R<T>(p->Oz) - R<T>(p->dz)));
    w.text("SPACING %8.12f %8.12f %8.12f\n", (double)(T)(R<T>(p->Lx) / (T)(nx - 1)),
           (double)(T)(R<T>(p->Ly) / (T)(ny - 1)), (double)(T)(R<T>(p->Lz) / (T)(nz - 1)));
    w.text("POINT_DATA %9i\n", (nx + 2) * (ny + 2) * (nz + 2));
    w.text("VECTORS bfield %s\n", real_str<T>());
    const size_t G = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
    for (size_t q = 0; q < 3 * G; q++) w.real(B0[q]);
    w.flush();
    const bool ok = w.ok && fclose(f) == 0;
    return ok ? GM_OK : gm::fail(GM_EIO, std::string("error: could not write '") + path + "'");
}

template <typename T>
int write_dump(const gm_params* p, const char* path, double t, double dt, const T* xb, const T* B, const T* J,
               const T* D, const T* cellVol, const T* convexity, const T* wedgeMin, const T* u) {
    if ((p->dumpJ && !J) || (p->dumpDetJac && !D) || (p->dumpCellVol && !cellVol) ||
        (p->dumpConvexity && !convexity) || (p->dumpWedgeMin && !wedgeMin) || !xb || !B || (p->inertia && !u))
        return gm::fail(GM_EPARAM, "gm_io_write_dump: a field selected by the dump flags is NULL");
    FILE* f = fopen(path, "wb");
    if (!f) return gm::fail(GM_EIO, std::string("error: could not open file '") + path + "'");
    Writer<T> w(f);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const int G = (nx + 2) * (ny + 2) * (nz + 2);
    const char* rs = real_str<T>();
    w.text("# vtk DataFile Version 2.0\n");
    w.text("GLEMuR data dump\n");
    w.text("BINARY\n");
    w.text("DATASET STRUCTURED_GRID\n");
    w.text("DIMENSIONS %9i %9i %9i\n", nx + 2, ny + 2, nz + 2);
    // parameters as field data (writeParams, io.cu:503-538)
    w.text("FIELD parameters %i\n", 9);
    w.text("t 1 1 %s\n", rs);
    w.real(t);
    w.text("dt 1 1 %s\n", rs);
    w.real(dt);
    w.text("nx_ny_nz 1 3 int\n");
    w.i32(nx); w.i32(ny); w.i32(nz);
    w.text("Lx_Ly_Lz 1 3 %s\n", rs);
    w.real(p->Lx); w.real(p->Ly); w.real(p->Lz);
    w.text("Ox_Oy_Oz 1 3 %s\n", rs);
    w.real(p->Ox); w.real(p->Oy); w.real(p->Oz);
    w.text("dx_dy_dz 1 3 %s\n", rs);
    w.real(p->dx); w.real(p->dy); w.real(p->dz);
    w.text("ampl 1 1 %s\n", rs);
    w.real(p->ampl);
    w.text("phi1_phi2 1 2 %s\n", rs);
    w.real(p->phi1); w.real(p->phi2);
    w.text("maxError 1 1 %s\n", rs);
    w.real(p->maxError);
    w.text("POINTS %9i %s\n", G, rs);
    for (size_t q = 0; q < 3 * (size_t)G; q++) w.real(xb[q]);
    w.text("POINT_DATA %9i\n", G);
    w.text("VECTORS bfield %s\n", rs);
    for (size_t q = 0; q < 3 * (size_t)G; q++) w.real(B[q]);
    auto ghost = [&](int i, int j, int k) { return i == 0 || i == nx + 1 || j == 0 || j == ny + 1 || k == 0 || k == nz + 1; };
    auto inner = [&](int i, int j, int k) { return (size_t)(i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k - 1)); };
    if (p->inertia) {
        // velocity, zero on the ghost layer (io.cu:269-291)
        w.text("VECTORS ufield %s\n", rs);
        for (int k = 0; k < nz + 2; k++)
            for (int j = 0; j < ny + 2; j++)
                for (int i = 0; i < nx + 2; i++)
                    for (int l = 0; l < 3; l++) w.real(ghost(i, j, k) ? 0.0 : (double)u[3 * inner(i, j, k) + l]);
    }
    if (p->dumpJ) {
        w.text("VECTORS jfield %s\n", rs);
        for (int k = 0; k < nz + 2; k++)
            for (int j = 0; j < ny + 2; j++)
                for (int i = 0; i < nx + 2; i++)
                    for (int l = 0; l < 3; l++) w.real(ghost(i, j, k) ? 0.0 : (double)J[3 * inner(i, j, k) + l]);
    }
    if (p->dumpDetJac) {
        w.text("SCALARS detJac %s\n", rs);
        w.text("LOOKUP_TABLE default\n");
        for (int q = 0; q < G; q++) w.real(D[q]);
    }
    const T* sc[3] = {cellVol, convexity, wedgeMin};
    const int32_t want[3] = {p->dumpCellVol, p->dumpConvexity, p->dumpWedgeMin};
    const char* names[3] = {"cellVol", "convexity", "wedgeMin"};
    for (int s = 0; s < 3; s++) {
        if (!want[s]) continue;
        w.text("SCALARS %s %s\n", names[s], rs);
        w.text("LOOKUP_TABLE default\n");
        for (int k = 0; k < nz + 2; k++)
            for (int j = 0; j < ny + 2; j++)
                for (int i = 0; i < nx + 2; i++)
                    w.real(ghost(i, j, k) ? 0.0 : (double)sc[s][inner(i, j, k)]);
    }
    w.flush();
    const bool ok = w.ok && fclose(f) == 0;
    return ok ? GM_OK : gm::fail(GM_EIO, std::string("error: could not write '") + path + "'");
}

bool read_line(FILE* f, std::string& line) {
    char b[256];
    if (!fgets(b, sizeof b, f)) return false;
    line = b;
    return true;
}

// readState (io.cu:390-499).  The parameter fields are matched by name as
// the reference does; t and dt are kept, the others are read past (the
// reference stores them into a by-value copy of its parameters, so they have
// no effect).  A field the reference does not name (maxError) is skipped by
// its declared size.
template <typename T>
int read_state(const gm_params* p, const char* save_path, const char* b0_path, T* xb, T* B0, double* t, double* dt,
               T* u) {
    FILE* f = fopen(save_path, "rb");
    if (!f) return gm::fail(GM_EIO, std::string("error: could not open file '") + save_path + "'");
    std::string line;
    const size_t G = (size_t)(p->nx + 2) * (p->ny + 2) * (p->nz + 2);
    auto bad = [&](const std::string& why) {
        fclose(f);
        return gm::fail(GM_EIO, std::string("error: ") + save_path + ": " + why);
    };
    for (int q = 0; q < 5; q++)
        if (!read_line(f, line)) return bad("truncated header");
    if (!read_line(f, line) || line.size() < 19) return bad("no FIELD line");
    const int numParams = atoi(line.substr(17, 2).c_str());
    bool have_t = false, have_dt = false;
    for (int q = 0; q < numParams; q++) {
        if (!read_line(f, line)) return bad("truncated parameter fields");
        const size_t sp = line.find(' ');
        const std::string name = line.substr(0, sp);
        int ncomp = 0, ntup = 0;
        char type[32] = {0};
        if (sscanf(line.c_str() + sp, "%d %d %31s", &ncomp, &ntup, type) != 3) return bad("bad field line");
        const size_t es = strcmp(type, "int") == 0 ? 4 : (strcmp(type, "float") == 0 ? 4 : 8);
        std::vector<unsigned char> v((size_t)ncomp * ntup * es);
        if (fread(v.data(), 1, v.size(), f) != v.size()) return bad("truncated field data");
        if ((name == "t" || name == "dt") && es == sizeof(T)) {
            T x;
            get_be(v.data(), &x);
            if (name == "t") { *t = (double)x; have_t = true; }
            else { *dt = (double)x; have_dt = true; }
        }
    }
    if (!have_t || !have_dt) return bad("t or dt missing");
    if (!read_line(f, line) || line.compare(0, 6, "POINTS") != 0) return bad("no POINTS line");
    std::vector<unsigned char> raw(3 * G * sizeof(T));
    if (fread(raw.data(), 1, raw.size(), f) != raw.size()) return bad("truncated grid data");
    for (size_t q = 0; q < 3 * G; q++) get_be(raw.data() + q * sizeof(T), &xb[q]);
    if (p->inertia) {
        // the velocity follows B (io.cu:466-481).  The reference reads one
        // text line, then 3G values from the "VECTORS bfield" line on, then one
        // more text line: that lands on the velocity block only when the last
        // bytes of the B block hold no newline byte.  Here each text line and
        // data block is read in turn.
        if (!read_line(f, line) || line.compare(0, 10, "POINT_DATA") != 0) return bad("no POINT_DATA line");
        if (!read_line(f, line) || line.compare(0, 14, "VECTORS bfield") != 0) return bad("no bfield");
        if (fread(raw.data(), 1, raw.size(), f) != raw.size()) return bad("truncated bfield");
        if (!read_line(f, line) || line.compare(0, 14, "VECTORS ufield") != 0) return bad("no ufield");
        if (fread(raw.data(), 1, raw.size(), f) != raw.size()) return bad("truncated ufield");
        const int nx = p->nx, ny = p->ny, nz = p->nz;
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++)
                    for (int l = 0; l < 3; l++) {
                        const size_t g = (size_t)(i + 1) + (size_t)(nx + 2) * ((j + 1) + (size_t)(ny + 2) * (k + 1));
                        get_be(raw.data() + (3 * g + l) * sizeof(T),
                               &u[l + 3 * ((size_t)i + (size_t)nx * (j + (size_t)ny * k))]);
                    }
    }
    fclose(f);
    f = fopen(b0_path, "rb");
    if (!f) return gm::fail(GM_EIO, std::string("error: could not open file '") + b0_path + "'");
    for (int q = 0; q < 9; q++)
        if (!read_line(f, line)) {
            fclose(f);
            return gm::fail(GM_EIO, std::string("error: ") + b0_path + ": truncated header");
        }
    if (fread(raw.data(), 1, raw.size(), f) != raw.size()) {
        fclose(f);
        return gm::fail(GM_EIO, std::string("error: ") + b0_path + ": truncated data");
    }
    for (size_t q = 0; q < 3 * G; q++) get_be(raw.data() + q * sizeof(T), &B0[q]);
    fclose(f);
    return GM_OK;
}

// One time-series line, writeTs (io.cu:542-678).
template <typename T>
int ts_line(const gm_params* p, const gm_reduction* r, double B2res, double t, double dt, int it, double maxDelta,
            int header, int toFile, char* buf, int size) {
    std::string s;
    char tmp[64];
    auto col = [&](bool on, const char* name, double v) {
        if (!on) return;
        if (header) snprintf(tmp, sizeof tmp, "%13s", name);
        else snprintf(tmp, sizeof tmp, "%12.5e ", (double)(T)v);
        s += tmp;
    };
    const bool in = p->inertia != 0;
    if (header) {
        snprintf(tmp, sizeof tmp, "#%7s", "it"); s += tmp;
        snprintf(tmp, sizeof tmp, "%13s", "t"); s += tmp;
        snprintf(tmp, sizeof tmp, "%13s", "dt"); s += tmp;
        snprintf(tmp, sizeof tmp, "%13s", toFile ? "maxDelta" : "maxError"); s += tmp;
    } else {
        snprintf(tmp, sizeof tmp, "%8i ", it); s += tmp;
        snprintf(tmp, sizeof tmp, "%12.5e ", (double)(T)t); s += tmp;
        snprintf(tmp, sizeof tmp, "%12.5e ", (double)(T)dt); s += tmp;
        snprintf(tmp, sizeof tmp, "%12.5e ", (double)(T)maxDelta); s += tmp;
    }
    const gm_reduction z = {};
    const gm_reduction& R = r ? *r : z;
    col(p->redJMax, "JMax", R.JMax);
    col(p->redJxB_B2Max, "JxB_B2Max", R.JxB_B2Max);
    col(p->redEpsilonStar, "epsilonStar", R.epsilonStar);
    col(p->redErrB_1ez, "errB_1ez", R.errB_1ez);
    col(p->redErrXb_XbAn, "errXb_XbAn", R.errXb_XbAn);
    col(p->redB2, "B2", R.B2);
    col(p->redB2f, "B2f", (double)((T)R.B2 - (T)B2res));
    col(p->redConvex, "convex", R.convex);
    col(p->redWedgeMin, "wedgeMin", R.wedgeMin);
    col(p->redU2 && in, "U2", R.U2);
    col(p->redUMax && in, "UMax", R.UMax);
    s += "\n";
    if ((int)s.size() + 1 > size) return gm::fail(GM_EPARAM, "gm_io_ts_line: buffer too small");
    memcpy(buf, s.c_str(), s.size() + 1);
    return (int)s.size();
}

}  // namespace

extern "C" {

int gm_device_count(int* n) {
    if (!n) return gm::fail(GM_EPARAM, "gm_device_count: null argument");
    *n = 0;
    const cudaError_t e = cudaGetDeviceCount(n);
    if (e != cudaSuccess) {
        *n = 0;
        return gm::fail(GM_ECUDA, std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
    }
    return GM_OK;
}

int gm_set_device(int dev) {
    const cudaError_t e = cudaSetDevice(dev);
    return e == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
}

int gm_io_write_cuda_info(const char* path, int precision, long activeDevice) {
    if (!path) return gm::fail(GM_EPARAM, "gm_io_write_cuda_info: null path");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) return gm::fail(GM_EIO, "error: could not locate CUDA devices");
    FILE* fd = fopen(path, "w");
    if (!fd) return gm::fail(GM_EIO, std::string("error: could not open file '") + path + "'");
    fprintf(fd, "number of CUDA devices: %i\n\n", count);
    fprintf(fd, "active device: %li\n\n", activeDevice);
    fprintf(fd, "PRECISION = %i\n\n", precision);
    for (int dev = 0; dev < count; dev++) {
        cudaDeviceProp d;
        if (cudaGetDeviceProperties(&d, dev) != cudaSuccess) {
            fclose(fd);
            return gm::fail(GM_EIO, "error: could not obtain device properties for device number " + std::to_string(dev));
        }
        // five properties left cudaDeviceProp in CUDA 13; the same values
        // come from device attributes
        int clock = 0, overlap = 0, timeout = 0, mode = 0, memclock = 0;
        cudaDeviceGetAttribute(&clock, cudaDevAttrClockRate, dev);
        cudaDeviceGetAttribute(&overlap, cudaDevAttrGpuOverlap, dev);
        cudaDeviceGetAttribute(&timeout, cudaDevAttrKernelExecTimeout, dev);
        cudaDeviceGetAttribute(&mode, cudaDevAttrComputeMode, dev);
        cudaDeviceGetAttribute(&memclock, cudaDevAttrMemoryClockRate, dev);
        fprintf(fd, "device number                   %i\n", dev);
        fprintf(fd, "name                            %s\n", d.name);
        fprintf(fd, "global memory [bytes]           %lu\n", (unsigned long)d.totalGlobalMem);
        fprintf(fd, "shared memory per block [bytes] %lu\n", (unsigned long)d.sharedMemPerBlock);
        fprintf(fd, "registers per block             %d\n", d.regsPerBlock);
        fprintf(fd, "threads per warp                %d\n", d.warpSize);
        fprintf(fd, "max memory pitch [bytes]        %lu\n", (unsigned long)d.memPitch);
        fprintf(fd, "max threads per block           %d\n", d.maxThreadsPerBlock);
        fprintf(fd, "max threads per block in x      %d\n", d.maxThreadsDim[0]);
        fprintf(fd, "max threads per block in y      %d\n", d.maxThreadsDim[1]);
        fprintf(fd, "max threads per block in z      %d\n", d.maxThreadsDim[2]);
        fprintf(fd, "max blocks per grid in x        %d\n", d.maxGridSize[0]);
        fprintf(fd, "max blocks per grid in y        %d\n", d.maxGridSize[1]);
        fprintf(fd, "max blocks per grid in z        %d\n", d.maxGridSize[2]);
        fprintf(fd, "clock rate [kHz]                %d\n", clock);
        fprintf(fd, "constant memory [bytes]         %lu\n", (unsigned long)d.totalConstMem);
        fprintf(fd, "compute capability major        %d\n", d.major);
        fprintf(fd, "compute capability minor        %d\n", d.minor);
        fprintf(fd, "texture alignment               %lu\n", (unsigned long)d.textureAlignment);
        fprintf(fd, "device overlap                  %d\n", overlap);
        fprintf(fd, "multiprocessors                 %d\n", d.multiProcessorCount);
        fprintf(fd, "kernel exec timeout             %d\n", timeout);
        fprintf(fd, "integrated GPU                  %d\n", d.integrated);
        fprintf(fd, "can map host memory             %d\n", d.canMapHostMemory);
        fprintf(fd, "computing mode                  %d\n", mode);
        fprintf(fd, "max size 1D textures            %d\n", d.maxTexture1D);
        fprintf(fd, "max size 2D textures in x       %d\n", d.maxTexture2D[0]);
        fprintf(fd, "max size 2D textures in y       %d\n", d.maxTexture2D[1]);
        fprintf(fd, "max size 3D textures in x       %d\n", d.maxTexture3D[0]);
        fprintf(fd, "max size 3D textures in y       %d\n", d.maxTexture3D[1]);
        fprintf(fd, "max size 3D textures in z       %d\n", d.maxTexture3D[2]);
        fprintf(fd, "concurrent kernels              %d\n", d.concurrentKernels);
        fprintf(fd, "ECC enabled                     %d\n", d.ECCEnabled);
        fprintf(fd, "PCI bus ID                      %d\n", d.pciBusID);
        fprintf(fd, "PCI device ID                   %d\n", d.pciDeviceID);
        fprintf(fd, "PCI domain ID                   %d\n", d.pciDomainID);
        fprintf(fd, "TCC drive                       %d\n", d.tccDriver);
        fprintf(fd, "asynchronous engine count       %d\n", d.asyncEngineCount);
        fprintf(fd, "unified addressing with host    %d\n", d.unifiedAddressing);
        fprintf(fd, "memory clock rate [kHz]         %d\n", memclock);
        fprintf(fd, "memory bus width [bits]         %d\n", d.memoryBusWidth);
        fprintf(fd, "l2 cache size [bytes]           %d\n", d.l2CacheSize);
        fprintf(fd, "maximum threads per multiproc.  %d\n", d.maxThreadsPerMultiProcessor);
        fprintf(fd, "\n");
    }
    return fclose(fd) == 0 ? GM_OK : gm::fail(GM_EIO, std::string("error: could not write '") + path + "'");
}

int gm_io_write_b0(const gm_params* p, const char* path, const void* B0) {
    if (!p || !path || !B0) return gm::fail(GM_EPARAM, "gm_io_write_b0: null argument");
    return p->precision == 32 ? write_b0<float>(p, path, (const float*)B0) : write_b0<double>(p, path, (const double*)B0);
}

int gm_io_write_dump(const gm_params* p, const char* path, double t, double dt, const void* xb, const void* B,
                     const void* J, const void* detJac, const void* cellVol, const void* convexity,
                     const void* wedgeMin, const void* u) {
    if (!p || !path) return gm::fail(GM_EPARAM, "gm_io_write_dump: null argument");
    if (p->precision == 32)
        return write_dump<float>(p, path, t, dt, (const float*)xb, (const float*)B, (const float*)J,
                                 (const float*)detJac, (const float*)cellVol, (const float*)convexity,
                                 (const float*)wedgeMin, (const float*)u);
    return write_dump<double>(p, path, t, dt, (const double*)xb, (const double*)B, (const double*)J,
                              (const double*)detJac, (const double*)cellVol, (const double*)convexity,
                              (const double*)wedgeMin, (const double*)u);
}

int gm_io_read_state(const gm_params* p, const char* save_path, const char* b0_path, void* xb, void* B0,
                     double* t, double* dt, void* u) {
    if (!p || !save_path || !b0_path || !xb || !B0 || !t || !dt || (p->inertia && !u))
        return gm::fail(GM_EPARAM, "gm_io_read_state: null argument");
    return p->precision == 32 ? read_state<float>(p, save_path, b0_path, (float*)xb, (float*)B0, t, dt, (float*)u)
                              : read_state<double>(p, save_path, b0_path, (double*)xb, (double*)B0, t, dt, (double*)u);
}

int gm_io_ts_line(const gm_params* p, const gm_reduction* r, double B2res, double t, double dt, int it,
                  double maxDelta, int header, int toFile, char* buf, int bufSize) {
    if (!p || !buf || bufSize <= 0) return gm::fail(GM_EPARAM, "gm_io_ts_line: null argument");
    return p->precision == 32 ? ts_line<float>(p, r, B2res, t, dt, it, maxDelta, header, toFile, buf, bufSize)
                              : ts_line<double>(p, r, B2res, t, dt, it, maxDelta, header, toFile, buf, bufSize);
}

}  // extern "C"
