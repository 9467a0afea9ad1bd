// glemur_main.cpp -- the `glemur` run-directory executable over the C-ABI.
//
// Same process contract as the reference's src/main.cu:44-394: run in a
// directory holding params.in and data/, optional `-d <device>`, writes
// cuda.info, data/B0.vtk, data/time_series.dat, data/dump<n>.vtk and
// data/save.vtk, prints the progress rows, restarts from data/save.vtk when
// fRestart is set, and ends with "glemur terminated successfully".  The
// reference picks its REAL type at compile time (src/Makefile:11, default
// 64); here `-p 32|64` picks it at run time (default 64).
//
// The loop of main.cu:259-384 runs on the device (gm_run_events); the host
// only wakes for the steps whose output is due: the time-series cadence nTs,
// the dtDump / dtSave crossings and the last step.
#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "glemur.h"

namespace {

int fail(const char* what) {
    printf("error: %s: %s\n", what, gm_last_error());
    return -1;
}

bool starts(const char* s, const char* pfx) { return strncmp(s, pfx, strlen(pfx)) == 0; }

// initResiduals (src/init.cu:13-26) in REAL; other initial fields leave it
// unset in the reference, here 0.
template <typename T>
double b2res(const gm_params& p) {
    if (starts(p.bInit, "Pontin09 ") || starts(p.bInit, "analytic ") || starts(p.bInit, "homZ ") ||
        starts(p.bInit, "blobs "))
        return (double)((T)1 * (T)p.Lx * (T)p.Ly * (T)p.Lz * (T)p.ampl);
    if (starts(p.bInit, "Borromean ")) return (double)((T)1 * (T)p.Lx * (T)p.Ly * (T)p.Lz * (T)p.bGround);
    return 0.0;
}

// ceil((t - dt) / dtDump) in REAL (main.cu:367-374).
template <typename T>
int dump_number(double t, double dt, double dtDump) {
    return (int)ceil((T)((T)t - (T)dt) / (T)dtDump);
}

struct TsFile {
    const gm_params* p;
    int append(const char* mode, const char* text) {
        FILE* f = fopen("data/time_series.dat", mode);
        if (!f) {
            printf("error: could not open file 'data/time_series.dat'\n");
            return -1;
        }
        fputs(text, f);
        fclose(f);
        return 0;
    }
};

template <typename T>
int run(gm_params& p, long activeDevice) {
    const size_t G = (size_t)(p.nx + 2) * (p.ny + 2) * (p.nz + 2);
    const size_t N = (size_t)p.nx * p.ny * p.nz;
    std::vector<T> B0(3 * G), xb(3 * G), B(3 * G), J(3 * N), D(G), cv(N), cx(N), wm(N), u(3 * N);
    (void)activeDevice;
    gm_handle* h = nullptr;
    if (gm_create(&p, &h)) return fail("could not set up the device state");
    double t = 0, dt = p.dt0;
    char line[4096];
    TsFile ts{&p};
    const double B2r = b2res<T>(p);
    if (!p.fRestart) {
        remove("data/save.vtk");
        if (gm_init_state(&p, B0.data(), xb.data())) return fail("initial state");
        if (gm_io_write_b0(&p, "data/B0.vtk", B0.data())) return fail("could not write data/B0.vtk");
        dt = (double)(T)p.dt0;
        t = 0;
        // writeTs at t = 0: the header, on stdout ("maxError") and as the new file ("maxDelta")
        if (gm_io_ts_line(&p, nullptr, B2r, 0, dt, 0, 0, 1, 0, line, sizeof line) < 0) return fail("time series");
        fputs(line, stdout);
        if (gm_io_ts_line(&p, nullptr, B2r, 0, dt, 0, 0, 1, 1, line, sizeof line) < 0) return fail("time series");
        if (ts.append("w+", line)) return -1;
    } else {
        if (gm_io_read_state(&p, "data/save.vtk", "data/B0.vtk", xb.data(), B0.data(), &t, &dt,
                             p.inertia ? u.data() : nullptr))
            return fail("could not read the restart state");
    }
    if (gm_upload(h, xb.data(), B0.data(), t, dt)) return fail("could not copy the state to the device");
    if (p.inertia && p.fRestart && gm_upload_u(h, u.data())) return fail("could not copy the velocity to the device");
    // the stage kernel's tile depth, timed once on this state (results do not depend on it)
    if (gm_autotune(h, 2, nullptr, nullptr)) return fail("autotuning failed");

    gm_state s;
    memset(&s, 0, sizeof s);
    for (;;) {
        if (gm_run_events(h, p.nCycle, &s)) {
            fail("time stepping stopped");
            gm_destroy(h);
            return -1;
        }
        if (!s.event) break;
        const int it = s.timeIndex - 1;    // main.cu's loop index of this step
        gm_reduction red;
        memset(&red, 0, sizeof red);
        // the post-accept B and J refresh (main.cu:342-353), then reductions
        if (gm_refresh(h, &red)) return fail("refresh");
        if (s.event & GM_EV_TS) {
            if (gm_io_ts_line(&p, &red, B2r, s.t, s.dtUsed, it, s.maxDelta, 0, 0, line, sizeof line) < 0)
                return fail("time series");
            fputs(line, stdout);
            if (ts.append("a", line)) return -1;
        }
        if (s.event & (GM_EV_DUMP | GM_EV_SAVE | GM_EV_LAST)) {
            // prepareDump (diagnostics.cu:138-212), then dumpState with the adapted dt
            if (gm_download(h, xb.data(), B.data(), J.data(), D.data())) return fail("download");
            if (p.inertia && gm_download_u(h, 5, u.data())) return fail("download");
            if (p.dumpCellVol || p.dumpConvexity || p.dumpWedgeMin)
                if (gm_grid_fields(h, cv.data(), cx.data(), wm.data())) return fail("grid fields");
            if (s.event & GM_EV_DUMP) {
                char name[64];
                snprintf(name, sizeof name, "data/dump%d.vtk", dump_number<T>(s.t, s.dt, p.dtDump));
                if (gm_io_write_dump(&p, name, s.t, s.dt, xb.data(), B.data(), J.data(), D.data(), cv.data(),
                                     cx.data(), wm.data(), u.data()))
                    return fail("dump");
            }
            if (s.event & (GM_EV_SAVE | GM_EV_LAST))
                if (gm_io_write_dump(&p, "data/save.vtk", s.t, s.dt, xb.data(), B.data(), J.data(), D.data(),
                                     cv.data(), cx.data(), wm.data(), u.data()))
                    return fail("save");
        }
    }
    if ((T)s.dt < (T)p.dtMin) printf("dt < dtMin = %e, stopping simulation\n", p.dtMin);
    gm_destroy(h);
    return 0;
}

}  // namespace

int main(int argc, char* argv[]) {
    int precision = 64;
    long activeDevice = 0;
    int deviceCount = 0;
    // -p is parsed first so the banner shows the run precision
    for (int a = 1; a + 1 < argc; a++)
        if (strcmp(argv[a], "-p") == 0) precision = atoi(argv[a + 1]);
    printf("GLEMuR\n\n");
    printf("PRECISION = %i\n", precision);
    if (precision != 32 && precision != 64) {
        printf("error: precision must be 32 or 64\n");
        return -1;
    }
    if (gm_device_count(&deviceCount) != GM_OK) {
        printf("error: could not locate CUDA devices\n");
        return -1;
    }
    if (deviceCount == 0) {
        printf("error: there are no CUDA compatible devices on this machine\n");
        return -1;
    }
    printf("CUDA device count = %i\n", deviceCount);
    int c;
    while ((c = getopt(argc, argv, "d:p:")) != -1) {
        if (c == 'd') {
            activeDevice = strtol(optarg, NULL, 10);
            if (activeDevice == 0 && optarg[0] != '0') {
                printf("error: device number is not integer\n");
                return -1;
            }
            if (activeDevice > deviceCount - 1 || activeDevice < 0) {
                printf("error: device number is not valid\n");
                return -1;
            }
        }
    }
    gm_set_device((int)activeDevice);
    printf("running on device %li\n", activeDevice);
    if (gm_io_write_cuda_info("cuda.info", precision, activeDevice)) {
        printf("error: could not write device properties into cuda.info\n");
        return -1;
    }
    const unsigned one = 1;
    printf(*(const unsigned char*)&one == 1 ? "endian = little\n" : "endian = big\n");
    printf(precision == 64 ? "bank size = 8 bytes\n" : "bank size = 4 bytes\n");

    gm_params p;
    if (gm_params_read(&p, "params.in", precision)) {
        printf("error: could not read params.in: %s\n", gm_last_error());
        return -1;
    }
    printf("jMethod = %s\n", p.jMethod);
    if (!starts(p.jMethod, "Stokes ") && !starts(p.jMethod, "Classic ") && !starts(p.jMethod, "Stokes4th ") &&
        !starts(p.jMethod, "StokesQuint ") && !starts(p.jMethod, "StokesTri ")) {
        printf("error: invalid method for computing J: %s\n", p.jMethod);
        return -1;
    }
    printf("initial B: %s\n", p.bInit);
    if (p.inertia) printf("initial U: %s\n", p.uInit);
    if (p.pressure) printf("include pressure gradient with beta = %f\n", p.beta);
    printf("tiles = 32 x 8 columns, one launch per Runge-Kutta stage, step loop on the device\n");
    const int rc = precision == 32 ? run<float>(p, activeDevice) : run<double>(p, activeDevice);
    if (rc) return rc;
    printf("glemur terminated successfully\n");
    return 0;
}
