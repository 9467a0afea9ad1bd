// ref_kernels.cu -- ORACLE: test infrastructure only.
//
// One translation unit that compiles the reference's own device kernels
// (src/maths.cu, boundaries.cu, current.cu, gradP.cu, rungeKutta.cu of
// SimonCan/glemur) into a cubin, unchanged, from where they lie in the
// reference tree (passed with -I).  The reference defines its __constant__
// parameter and Runge-Kutta coefficient symbols in src/main.cu:34-38, which is
// host code and not compiled here, so they are defined below with the
// declarations of src/global.h:168-172.
//
// Built only where the reference tree exists (oracle/build.py); the
// cubin is loaded by ref_launcher.cpp through the CUDA driver API.
#include "global.h"

__constant__ Parameters dev_params;
__constant__ REAL a_i[6];
__constant__ REAL b_ij[7 * 6];
__constant__ REAL c_i[6];
__constant__ REAL cs_i[6];

#include "maths.cu"
#include "boundaries.cu"
#include "current.cu"
#include "gradP.cu"
#include "rungeKutta.cu"
