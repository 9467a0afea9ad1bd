// gm_kernels_impl.cuh -- kernel bodies; included once per precision by
// gm_kernels_f32.cu and gm_kernels_f64.cu.
#pragma once

#include <float.h>
#include <math.h>

#include "glemur.h"
#include "gm_kernels.cuh"

namespace gmk {

__device__ __forceinline__ long long gidx(int px, int py, int i, int j, int k) {
    return (long long)(i + 2) + (long long)px * ((long long)(j + 2) + (long long)py * (long long)(k + 2));
}

template <typename T>
__device__ __forceinline__ T det3(const T j[3][3]) {
    return j[0][0] * j[1][1] * j[2][2] + j[0][1] * j[1][2] * j[2][0] + j[0][2] * j[1][0] * j[2][1] -
           j[0][0] * j[1][2] * j[2][1] - j[0][1] * j[1][0] * j[2][2] - j[0][2] * j[1][1] * j[2][0];
}

// Jacobian determinant.  In FP32 storage the determinant of a strongly
// sheared cell (cancellation among the six Sarrus products) is recomputed in
// double from the same single-precision Jacobian.
template <typename T>
__device__ __forceinline__ T det_guarded(const T j[3][3]) {
    T d = det3(j);
    if (sizeof(T) == 4) {
        T mag = fabs(j[0][0] * j[1][1] * j[2][2]) + fabs(j[0][1] * j[1][2] * j[2][0]) +
                fabs(j[0][2] * j[1][0] * j[2][1]) + fabs(j[0][0] * j[1][2] * j[2][1]) +
                fabs(j[0][1] * j[1][0] * j[2][2]) + fabs(j[0][2] * j[1][1] * j[2][0]);
        if (fabs(d) < (T)0.0625 * mag) {
            double jd[3][3];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) jd[a][b] = (double)j[a][b];
            d = (T)det3<double>(jd);
        }
    }
    return d;
}

// Correctly rounded reciprocal (the value of 1/x with IEEE division).
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }

template <typename T>
__device__ __forceinline__ void cross3(const T a[3], const T b[3], T c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// Shared-memory tile views: a ring of XR position planes (plane k in slot
// (k + OFF) % XR) and a ring of B planes.
template <typename T, int NB, int XR = XRING, int OFF = 10>
struct Tile {
    T* xs;
    T* bs;
    int i0, j0, HX, HY, BX, BY;
    int slot = 0;     // elements between position-plane slots (0: 3 * HY * HX)
    __device__ __forceinline__ T& x(int k, int c, int j, int i) const {
        const int ss = slot ? slot : 3 * HY * HX;
        return xs[((k + OFF) % XR) * ss + (c * HY + (j - j0 + 2)) * HX + (i - i0 + 2)];
    }
    __device__ __forceinline__ T& b(int k, int c, int j, int i) const {
        return bs[((((k + 10) % BRING) * NB + c) * BY + (j - j0 + 1)) * BX + (i - i0 + 1)];
    }
};

// B and Delta at an interior (or periodic-image) point: B_JacB0,
// src/rungeKutta.cu:79-106.
template <typename T, int NB>
__device__ __forceinline__ void b_interior(const KP<T>& p, const Tile<T, NB>& t, const T* __restrict__ B0, int i,
                                           int j, int k, T Bv[3], T* D) {
    T jac[3][3];
#pragma unroll
    for (int l = 0; l < 3; l++) {
        // (a - b) * d1 / 2 == (a - b) * (d1 / 2) exactly (scaling by 2)
        jac[l][0] = (t.x(k, l, j, i + 1) - t.x(k, l, j, i - 1)) * p.hdx1;
        jac[l][1] = (t.x(k, l, j + 1, i) - t.x(k, l, j - 1, i)) * p.hdy1;
        jac[l][2] = (t.x(k + 1, l, j, i) - t.x(k - 1, l, j, i)) * p.hdz1;
    }
    T det = det_guarded(jac);
    T detJac1 = rcp_rn(det);
    long long g = gidx(p.px, p.py, i, j, k);
    T b0 = __ldg(&B0[g]), b1 = __ldg(&B0[p.cs + g]), b2 = __ldg(&B0[2 * p.cs + g]);
#pragma unroll
    for (int l = 0; l < 3; l++) Bv[l] = (jac[l][0] * b0 + jac[l][1] * b1 + jac[l][2] * b2) * detJac1;
    *D = rcp_rn(detJac1);
}

// B and Delta on the ghost plane of a non-periodic face with normal axis a:
// updateBbound, src/boundaries.cu:39-446.  The outer plane is the ghost
// plane shifted by the grid spacing; in-plane neighbours at the edges of the
// reference's 16x16 launch blocks are the own position shifted by the
// spacing (boundaries.cu:72-109, 212-237, 340-365); B.n = B0.n.
// addDist, src/boundaries.cu:11-35: the initial distortion at inner column
// (i, j) and height z, component l (0: x, 1: y).  PI is a double constant, so
// in FP32 the sine's argument, the sine and the products are double and only
// the assignment to distX / distY rounds; the centerShift form takes exp in
// REAL and subtracts the double constant 0.15366.
template <typename T>
__device__ __forceinline__ T add_dist(const KP<T>& p, int i, int j, T z, int l) {
    const T x = p.dx * (T)i + p.Ox;
    const T y = p.dy * (T)j + p.Oy;
    T distX = 0, distY = 0;
    if (p.initDistCode == 0) {
        distY = (T)(-p.shA * sin(p.shK * (T)2 * 3.141592653589793 * (x + p.Ox - p.dx / (T)2) / (p.Lx + p.dx)) * z);
        distX = (T)(-p.shB * sin(p.shK * (T)2 * 3.141592653589793 * (distY + y + p.Oy - p.dy / (T)2) / (p.Ly + p.dy)) *
                    z);
    } else {
        distY = (T)(p.shA * exp(-p.shK * x * x) * ((T)1 - y * y) * (exp((T)-1 * z + (T)1) - 0.15366));
    }
    return l == 0 ? distX : distY;
}

template <typename T, bool SHEAR = true, class TileT>
__device__ __forceinline__ void b_face(const KP<T>& p, const TileT& t, const T* __restrict__ B0, int a, int i,
                                       int j, int k, T Bv[3], T* D) {
    const int u = (a == 0) ? 1 : 0;
    const int v = (a == 2) ? 1 : 2;
    int c3[3] = {i, j, k};
    const int n3[3] = {p.nx, p.ny, p.nz};
    const T d3[3] = {p.dx, p.dy, p.dz};
    const T d13[3] = {p.dx1, p.dy1, p.dz1};
    const int side = c3[a] < 0 ? 0 : 1;
    T X1[3], Xin[3], Xo[3], Lu[3], Ru[3], Lv[3], Rv[3];
    int ci[3] = {i, j, k};
    ci[a] = side ? n3[a] - 1 : 0;
#pragma unroll
    for (int l = 0; l < 3; l++) {
        X1[l] = t.x(k, l, j, i);
        Xin[l] = t.x(ci[2], l, ci[1], ci[0]);
        Xo[l] = X1[l];
    }
    Xo[a] = X1[a] + (side ? d3[a] : -d3[a]);
    const int iu = c3[u], iv = c3[v];
    int cl[3], cr[3];
#pragma unroll
    for (int q = 0; q < 3; q++) { cl[q] = c3[q]; cr[q] = c3[q]; }
    cl[u] -= 1;
    cr[u] += 1;
    const bool eLu = (iu % 16 == 0), eRu = (iu % 16 == 15) || (iu == n3[u] - 1);
#pragma unroll
    for (int l = 0; l < 3; l++) {
        Lu[l] = eLu ? X1[l] : t.x(cl[2], l, cl[1], cl[0]);
        Ru[l] = eRu ? X1[l] : t.x(cr[2], l, cr[1], cr[0]);
    }
    if (eLu) Lu[u] = X1[u] - d3[u];
    if (eRu) Ru[u] = X1[u] + d3[u];
#pragma unroll
    for (int q = 0; q < 3; q++) { cl[q] = c3[q]; cr[q] = c3[q]; }
    cl[v] -= 1;
    cr[v] += 1;
    const bool eLv = (iv % 16 == 0), eRv = (iv % 16 == 15) || (iv == n3[v] - 1);
#pragma unroll
    for (int l = 0; l < 3; l++) {
        Lv[l] = eLv ? X1[l] : t.x(cl[2], l, cl[1], cl[0]);
        Rv[l] = eRv ? X1[l] : t.x(cr[2], l, cr[1], cr[0]);
    }
    if (eLv) Lv[v] = X1[v] - d3[v];
    if (eRv) Rv[v] = X1[v] + d3[v];
    if (SHEAR && a == 2 && p.shear) {
        // an initially distorted grid: the outer ghost plane and the neighbours
        // extrapolated at the 16-wide block edges carry the distortion
        // (src/boundaries.cu:65-107).  The line-tied ghost planes do not move,
        // so these positions are constants of the run (k_shear_table).
        const T* tb = p.shearTab + 10 * ((long long)side * p.nx * p.ny + (long long)j * p.nx + i);
        Xo[0] = tb[0]; Xo[1] = tb[1];
        if (eLu) { Lu[0] = tb[2]; Lu[1] = tb[3]; }
        if (eRu) { Ru[0] = tb[4]; Ru[1] = tb[5]; }
        if (eLv) { Lv[0] = tb[6]; Lv[1] = tb[7]; }
        if (eRv) { Rv[0] = tb[8]; Rv[1] = tb[9]; }
    }
    T jac[3][3];
#pragma unroll
    for (int l = 0; l < 3; l++) {
        jac[l][u] = (Ru[l] - Lu[l]) * d13[u] / 2;
        jac[l][v] = (Rv[l] - Lv[l]) * d13[v] / 2;
        jac[l][a] = (side ? (Xo[l] - Xin[l]) : (Xin[l] - Xo[l])) * d13[a] / 2;
    }
    T detJac1 = rcp_rn(det_guarded(jac));
    long long g = gidx(p.px, p.py, i, j, k);
    T b0[3] = {__ldg(&B0[g]), __ldg(&B0[p.cs + g]), __ldg(&B0[2 * p.cs + g])};
#pragma unroll
    for (int l = 0; l < 3; l++) Bv[l] = (jac[l][0] * b0[0] + jac[l][1] * b0[1] + jac[l][2] * b0[2]) * detJac1;
    Bv[a] = b0[a];
    *D = rcp_rn(detJac1);
}

// Mimetic current: circulation of B around the three quadrilaterals through
// the face neighbours, area-weighted normals and a 3x3 solve; JStokes,
// src/current.cu:290-406.  Neighbour order: -x, +x, -y, +y, -z, +z.
// The circulations are accumulated without the 1/2 of the edge averages (so
// they come out doubled) and the normals without their 1/4 (so the inverse
// normal matrix comes out quartered); J = 2 * (quartered inverse) . (doubled
// circulations).  Power-of-two scalings leave every rounding unchanged.
template <typename T>
__device__ __forceinline__ void stokes(const T xn[6][3], const T bn[6][3], T J[3]) {
    constexpr int Q[3][4] = {{0, 2, 1, 3}, {2, 4, 3, 5}, {4, 0, 5, 1}};
    T NA[3][3], II[3];
#pragma unroll
    for (int qd = 0; qd < 3; qd++) {
        T dxv[4][3];
        T I = 0;
#pragma unroll
        for (int l = 0; l < 3; l++) {
#pragma unroll
            for (int c = 0; c < 4; c++) dxv[c][l] = xn[Q[qd][(c + 1) & 3]][l] - xn[Q[qd][c]][l];
            I += (bn[Q[qd][1]][l] + bn[Q[qd][0]][l]) * dxv[0][l] + (bn[Q[qd][2]][l] + bn[Q[qd][1]][l]) * dxv[1][l] +
                 (bn[Q[qd][3]][l] + bn[Q[qd][2]][l]) * dxv[2][l] + (bn[Q[qd][0]][l] + bn[Q[qd][3]][l]) * dxv[3][l];
        }
        T cr[4][3];
#pragma unroll
        for (int c = 0; c < 4; c++) cross3(dxv[c], dxv[(c + 1) & 3], cr[c]);
        II[qd] = I;
#pragma unroll
        for (int l = 0; l < 3; l++) NA[qd][l] = cr[0][l] + cr[1][l] + cr[2][l] + cr[3][l];
    }
    T detN1 = rcp_rn(det3(NA));
    T NA1[3][3];
    NA1[0][0] = (NA[1][1] * NA[2][2] - NA[1][2] * NA[2][1]) * detN1;
    NA1[0][1] = (NA[0][2] * NA[2][1] - NA[0][1] * NA[2][2]) * detN1;
    NA1[0][2] = (NA[0][1] * NA[1][2] - NA[0][2] * NA[1][1]) * detN1;
    NA1[1][0] = (NA[1][2] * NA[2][0] - NA[1][0] * NA[2][2]) * detN1;
    NA1[1][1] = (NA[0][0] * NA[2][2] - NA[0][2] * NA[2][0]) * detN1;
    NA1[1][2] = (NA[0][2] * NA[1][0] - NA[0][0] * NA[1][2]) * detN1;
    NA1[2][0] = (NA[1][0] * NA[2][1] - NA[1][1] * NA[2][0]) * detN1;
    NA1[2][1] = (NA[0][1] * NA[2][0] - NA[0][0] * NA[2][1]) * detN1;
    NA1[2][2] = (NA[0][0] * NA[1][1] - NA[0][1] * NA[1][0]) * detN1;
#pragma unroll
    for (int l = 0; l < 3; l++) J[l] = (NA1[l][0] * II[0] + NA1[l][1] * II[1] + NA1[l][2] * II[2]) * (T)2;
}

// Finite-difference current: JClassic, src/current.cu:10-218.  J = curl B
// for B = jac.B0 / Delta, differentiated by the chain rule on the initial
// grid: d B_m / d X_a = sum_b (d2x[m][a][b] B0_b / Delta + jac[m][b]
// dB0_b/dX_a / Delta + jac[m][b] B0_b d(1/Delta)/dX_a), and
// d / d x_c = sum_a jac^-1[a][c] d / d X_a.  Reads the positions of the
// point, its face and edge neighbours (the position ring), Delta at the point
// and its face neighbours (the B ring, ghost values included) and B0 there
// (global memory); B itself is not used.
template <typename T, class TileT>
__device__ __forceinline__ void j_classic(const KP<T>& p, const TileT& t, const T* __restrict__ B0, int i, int j,
                                          int k, T Jv[3]) {
    T jac[3][3], jac1[3][3], dB0[3][3], dDet1[3], B0l[3];
#define XV(di, dj, dk, l) t.x(k + (dk), l, j + (dj), i + (di))
#define B0V(di, dj, dk, l) __ldg(&B0[(long long)(l) * p.cs + gidx(p.px, p.py, i + (di), j + (dj), k + (dk))])
#define DV(di, dj, dk) t.b(k + (dk), 3, j + (dj), i + (di))
    const T det1 = rcp_rn(DV(0, 0, 0));
#pragma unroll
    for (int l = 0; l < 3; l++) {
        jac[l][0] = (XV(1, 0, 0, l) - XV(-1, 0, 0, l)) * p.dx1 / 2;
        jac[l][1] = (XV(0, 1, 0, l) - XV(0, -1, 0, l)) * p.dy1 / 2;
        jac[l][2] = (XV(0, 0, 1, l) - XV(0, 0, -1, l)) * p.dz1 / 2;
        B0l[l] = B0V(0, 0, 0, l);
        dB0[l][0] = (B0V(1, 0, 0, l) - B0V(-1, 0, 0, l)) * p.dx1 / 2;
        dB0[l][1] = (B0V(0, 1, 0, l) - B0V(0, -1, 0, l)) * p.dy1 / 2;
        dB0[l][2] = (B0V(0, 0, 1, l) - B0V(0, 0, -1, l)) * p.dz1 / 2;
    }
    jac1[0][0] = (jac[1][1] * jac[2][2] - jac[1][2] * jac[2][1]) * det1;
    jac1[0][1] = (jac[0][2] * jac[2][1] - jac[0][1] * jac[2][2]) * det1;
    jac1[0][2] = (jac[0][1] * jac[1][2] - jac[0][2] * jac[1][1]) * det1;
    jac1[1][0] = (jac[1][2] * jac[2][0] - jac[1][0] * jac[2][2]) * det1;
    jac1[1][1] = (jac[0][0] * jac[2][2] - jac[0][2] * jac[2][0]) * det1;
    jac1[1][2] = (jac[0][2] * jac[1][0] - jac[0][0] * jac[1][2]) * det1;
    jac1[2][0] = (jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0]) * det1;
    jac1[2][1] = (jac[0][1] * jac[2][0] - jac[0][0] * jac[2][1]) * det1;
    jac1[2][2] = (jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0]) * det1;
    dDet1[0] = (rcp_rn(DV(1, 0, 0)) - rcp_rn(DV(-1, 0, 0))) * p.dx1 / 2;
    dDet1[1] = (rcp_rn(DV(0, 1, 0)) - rcp_rn(DV(0, -1, 0))) * p.dy1 / 2;
    dDet1[2] = (rcp_rn(DV(0, 0, 1)) - rcp_rn(DV(0, 0, -1))) * p.dz1 / 2;
    Jv[0] = 0; Jv[1] = 0; Jv[2] = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        // second derivatives d2x[m][a][b] of the three components for this a
        T d2[3][3];
#pragma unroll
        for (int m = 0; m < 3; m++) {
            const T xc2 = 2 * XV(0, 0, 0, m);
            if (a == 0) {
                d2[m][0] = (XV(1, 0, 0, m) - xc2 + XV(-1, 0, 0, m)) * p.dx1 * p.dx1;
                d2[m][1] = (XV(1, 1, 0, m) - XV(1, -1, 0, m) - XV(-1, 1, 0, m) + XV(-1, -1, 0, m)) * p.dx1 * p.dy1 / 4;
                d2[m][2] = (XV(1, 0, 1, m) - XV(1, 0, -1, m) - XV(-1, 0, 1, m) + XV(-1, 0, -1, m)) * p.dx1 * p.dz1 / 4;
            } else if (a == 1) {
                d2[m][0] = (XV(1, 1, 0, m) - XV(1, -1, 0, m) - XV(-1, 1, 0, m) + XV(-1, -1, 0, m)) * p.dx1 * p.dy1 / 4;
                d2[m][1] = (XV(0, 1, 0, m) - xc2 + XV(0, -1, 0, m)) * p.dy1 * p.dy1;
                d2[m][2] = (XV(0, 1, 1, m) - XV(0, -1, 1, m) - XV(0, 1, -1, m) + XV(0, -1, -1, m)) * p.dy1 * p.dz1 / 4;
            } else {
                d2[m][0] = (XV(1, 0, 1, m) - XV(1, 0, -1, m) - XV(-1, 0, 1, m) + XV(-1, 0, -1, m)) * p.dx1 * p.dz1 / 4;
                d2[m][1] = (XV(0, 1, 1, m) - XV(0, -1, 1, m) - XV(0, 1, -1, m) + XV(0, -1, -1, m)) * p.dy1 * p.dz1 / 4;
                d2[m][2] = (XV(0, 0, 1, m) - xc2 + XV(0, 0, -1, m)) * p.dz1 * p.dz1;
            }
        }
#pragma unroll
        for (int b = 0; b < 3; b++) {
            T dB[3];
#pragma unroll
            for (int m = 0; m < 3; m++)
                dB[m] = d2[m][b] * B0l[b] * det1 + jac[m][b] * dB0[b][a] * det1 + jac[m][b] * B0l[b] * dDet1[a];
            Jv[0] += jac1[a][1] * dB[2] - jac1[a][2] * dB[1];
            Jv[1] += jac1[a][2] * dB[0] - jac1[a][0] * dB[2];
            Jv[2] += jac1[a][0] * dB[1] - jac1[a][1] * dB[0];
        }
    }
#undef XV
#undef B0V
#undef DV
}

// Pressure gradient grad(p) for p = p0(X)/Delta: gradPClassic,
// src/gradP.cu:91-155 (uniform p0 = beta), plus (1/Delta) J^-T grad_X p0 for
// a non-uniform p0(X) (no counterpart in the reference).
template <typename T, class TileT>
__device__ __forceinline__ void grad_p(const KP<T>& p, const TileT& t, int i, int j, int k, T D, T g[3]) {
    T jac[3][3], jac1[3][3];
    const T det1 = (T)1 / D;
#define XV(di, dj, dk, l) t.x(k + (dk), l, j + (dj), i + (di))
#pragma unroll
    for (int l = 0; l < 3; l++) {
        jac[l][0] = (XV(1, 0, 0, l) - XV(-1, 0, 0, l)) * p.dx1 / 2;
        jac[l][1] = (XV(0, 1, 0, l) - XV(0, -1, 0, l)) * p.dy1 / 2;
        jac[l][2] = (XV(0, 0, 1, l) - XV(0, 0, -1, l)) * p.dz1 / 2;
    }
    jac1[0][0] = (jac[1][1] * jac[2][2] - jac[1][2] * jac[2][1]) * det1;
    jac1[0][1] = (jac[0][2] * jac[2][1] - jac[0][1] * jac[2][2]) * det1;
    jac1[0][2] = (jac[0][1] * jac[1][2] - jac[0][2] * jac[1][1]) * det1;
    jac1[1][0] = (jac[1][2] * jac[2][0] - jac[1][0] * jac[2][2]) * det1;
    jac1[1][1] = (jac[0][0] * jac[2][2] - jac[0][2] * jac[2][0]) * det1;
    jac1[1][2] = (jac[0][2] * jac[1][0] - jac[0][0] * jac[1][2]) * det1;
    jac1[2][0] = (jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0]) * det1;
    jac1[2][1] = (jac[0][1] * jac[2][0] - jac[0][0] * jac[2][1]) * det1;
    jac1[2][2] = (jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0]) * det1;
    // grad_x(1/Delta) up to the factor 1/Delta: -sum_{a,b,l} d2x_a/dX_b dX_l
    // jac1[b][a] jac1[l][c] (gradP.cu:127-150), summed as
    // -sum_l v_l jac1[l][c] with v_l = sum_{a,b} d2x_a/dX_b dX_l jac1[b][a]
    // (36 products instead of 162; a different rounding order)
    T v[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        T d2[3][3];
        d2[0][0] = (XV(1, 0, 0, a) - 2 * XV(0, 0, 0, a) + XV(-1, 0, 0, a)) * p.dx1 * p.dx1;
        d2[1][1] = (XV(0, 1, 0, a) - 2 * XV(0, 0, 0, a) + XV(0, -1, 0, a)) * p.dy1 * p.dy1;
        d2[2][2] = (XV(0, 0, 1, a) - 2 * XV(0, 0, 0, a) + XV(0, 0, -1, a)) * p.dz1 * p.dz1;
        d2[0][1] = (XV(1, 1, 0, a) - XV(1, -1, 0, a) - XV(-1, 1, 0, a) + XV(-1, -1, 0, a)) * p.dx1 * p.dy1 / 4;
        d2[0][2] = (XV(1, 0, 1, a) - XV(1, 0, -1, a) - XV(-1, 0, 1, a) + XV(-1, 0, -1, a)) * p.dx1 * p.dz1 / 4;
        d2[1][2] = (XV(0, 1, 1, a) - XV(0, -1, 1, a) - XV(0, 1, -1, a) + XV(0, -1, -1, a)) * p.dy1 * p.dz1 / 4;
        d2[1][0] = d2[0][1];
        d2[2][0] = d2[0][2];
        d2[2][1] = d2[1][2];
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int l = 0; l < 3; l++) v[l] += d2[b][l] * jac1[b][a];
    }
    T acc[3];
#pragma unroll
    for (int c = 0; c < 3; c++) acc[c] = -(v[0] * jac1[0][c] + v[1] * jac1[1][c] + v[2] * jac1[2][c]);
#undef XV
    if (p.p0Amp != (T)0) {
        // p0(X) on the initial grid X = (dx i + Ox, dy j + Oy)
        const T X = p.dx * (T)i + p.Ox, Y = p.dy * (T)j + p.Oy;
        const T e = p.p0Amp * exp(-(X * X + Y * Y) * p.inv_p0W2);
        const T p0 = p.beta * ((T)1 + e);
        const T be2 = -2 * p.beta * e * p.inv_p0W2;
        const T dp0[3] = {be2 * X, be2 * Y, (T)0};
#pragma unroll
        for (int c = 0; c < 3; c++)
            g[c] = (p0 * acc[c] + dp0[0] * jac1[0][c] + dp0[1] * jac1[1][c] + dp0[2] * jac1[2][c]) * det1;
    } else {
#pragma unroll
        for (int c = 0; c < 3; c++) g[c] = acc[c] * (p.beta * det1);
    }
}

// Store a grid position and its periodic images (ghost layers 1 and 2), the
// images shifted by -/+ (L + d) as setGridPeriFace writes them
// (boundaries.cu:546-549, 561-564, 576-579).
template <typename T>
__device__ __forceinline__ void store_pos(const KP<T>& p, T* __restrict__ X, int i, int j, int k, const T v[3]) {
    int oi[3] = {0, 0, 0}, oj[3] = {0, 0, 0}, ok[3] = {0, 0, 0};
    int ni = 1, nj = 1, nk = 1;
    if (p.xPeri) { if (i < 2) oi[ni++] = 1; if (i >= p.nx - 2) oi[ni++] = -1; }
    if (p.yPeri) { if (j < 2) oj[nj++] = 1; if (j >= p.ny - 2) oj[nj++] = -1; }
    if (p.zPeri) { if (k < 2) ok[nk++] = 1; if (k >= p.nz - 2) ok[nk++] = -1; }
    for (int a = 0; a < ni; a++)
        for (int b = 0; b < nj; b++)
            for (int c = 0; c < nk; c++) {
                const int si = oi[a], sj = oj[b], sk = ok[c];
                T w0 = v[0], w1 = v[1], w2 = v[2];
                if (si > 0) w0 = (v[0] + p.Lx) + p.dx; else if (si < 0) w0 = (v[0] - p.Lx) - p.dx;
                if (sj > 0) w1 = (v[1] + p.Ly) + p.dy; else if (sj < 0) w1 = (v[1] - p.Ly) - p.dy;
                if (sk > 0) w2 = (v[2] + p.Lz) + p.dz; else if (sk < 0) w2 = (v[2] - p.Lz) - p.dz;
                long long g = gidx(p.px, p.py, i + si * p.nx, j + sj * p.ny, k + sk * p.nz);
                X[g] = w0;
                X[p.cs + g] = w1;
                X[2 * p.cs + g] = w2;
            }
}

__device__ __forceinline__ bool finite3d(double a, double b, double c) { return isfinite(a) && isfinite(b) && isfinite(c); }

template <typename T, bool PRESS, int MODE, bool LAST>
__global__ void __launch_bounds__(256) k_stage(const __grid_constant__ StageArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    constexpr int NB = 4;     // B and Delta (Delta: pressure, the Classic current, diagnostics)
    const KP<T>& p = a.p;
    DevState* st = a.st;
    if (MODE == MODE_STAGE && st->done) return;

    const int TY = blockDim.y;
    const int HX = TX + 4, HY = TY + 4, BX = TX + 2, BY = TY + 2;
    const int planeX = 3 * HY * HX, planeB = NB * BY * BX;
    Tile<T, NB> t;
    t.xs = reinterpret_cast<T*>(smraw);
    t.bs = t.xs + XRING * planeX;
    t.HX = HX; t.HY = HY; t.BX = BX; t.BY = BY;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx, nthr = TX * TY;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * a.TZ;
    t.i0 = i0; t.j0 = j0;
    const int kend = min(k0 + a.TZ, p.nz);
    const int cur = st->cur;
    const T* __restrict__ Xin = ((MODE == MODE_DIAG && !a.jpass) || a.n == 0) ? a.X[cur] : a.XS[(a.n - 1) & 1];
    const T dtT = (T)st->dt;
    const int n = a.n;
    const long long N = p.N;

    double dmax = 0;      // running max of the error norm (stage 5)
    bool bad = false;     // NaN/Inf seen
    // diagnostic partials
    double r_sum[7] = {0, 0, 0, 0, 0, 0, 0};
    double r_max[4] = {0, 0, 0, 0};
    double r_min[3] = {DBL_MAX, DBL_MAX, 1.0};

    for (int kk = k0 - 2; kk <= kend + 1; kk++) {
        // (a) positions of plane kk, tile + 2-point halo
        {
            T* dst = t.xs + ((kk + 10) % XRING) * planeX;
            const int area = HY * HX;
            for (int e = tid; e < planeX; e += nthr) {
                const int c = e / area;
                const int r = e - c * area;
                const int jj = r / HX, ii = r - jj * HX;
                const int gi = i0 - 2 + ii, gj = j0 - 2 + jj;
                if (gi < p.nx + 2 && gj < p.ny + 2 && kk >= -2 && kk < p.nz + 2)
                    dst[e] = Xin[c * p.cs + gidx(p.px, p.py, gi, gj, kk)];
            }
        }
        __syncthreads();
        // (b) B and Delta on plane kb = kk - 1: tile + face halo
        const int kb = kk - 1;
        if (kb >= k0 - 1) {
            T* bdst = t.bs + ((kb + 10) % BRING) * planeB;
            const bool zo = (kb < 0 || kb >= p.nz);
            for (int e = tid; e < BY * BX; e += nthr) {
                const int jj = e / BX, ii = e - jj * BX;
                const int i = i0 - 1 + ii, j = j0 - 1 + jj;
                const bool hx = (ii == 0 || ii == BX - 1), hy = (jj == 0 || jj == BY - 1);
                if (hx && hy) continue;
                if (i > p.nx || j > p.ny) continue;
                const bool xo = (i < 0 || i >= p.nx), yo = (j < 0 || j >= p.ny);
                if ((int)xo + (int)yo + (int)zo >= 2) continue;
                T Bv[3], D;
                int face = -1;
                if (zo && !p.zPeri) {
                    if (hx || hy) continue;      // only the tile points of a line-tied ghost plane are used
                    face = 2;
                } else if (xo && !p.xPeri) {
                    face = 0;
                } else if (yo && !p.yPeri) {
                    face = 1;
                }
                if (face >= 0) b_face<T>(p, t, a.B0, face, i, j, kb, Bv, &D);
                else b_interior<T, NB>(p, t, a.B0, i, j, kb, Bv, &D);
                bdst[(0 * BY + jj) * BX + ii] = Bv[0];
                bdst[(1 * BY + jj) * BX + ii] = Bv[1];
                bdst[(2 * BY + jj) * BX + ii] = Bv[2];
                if (NB == 4) bdst[(3 * BY + jj) * BX + ii] = D;
                if (MODE == MODE_DIAG && face >= 0) {
                    // ghost-plane B and Delta of a non-periodic face: owned by exactly one CTA
                    const bool own = (kb >= k0 && kb < kend) || (face == 2 && ((kb < 0 && k0 == 0) || (kb >= p.nz && kend == p.nz)));
                    const bool ownxy = (face == 2) || (face == 0 && j >= j0 && j < j0 + TY) || (face == 1 && i >= i0 && i < i0 + TX);
                    if (own && ownxy) {
                        const long long gq = (long long)(i + 1) + (long long)(p.nx + 2) * ((long long)(j + 1) + (long long)(p.ny + 2) * (kb + 1));
                        a.outB[3 * gq + 0] = Bv[0];
                        a.outB[3 * gq + 1] = Bv[1];
                        a.outB[3 * gq + 2] = Bv[2];
                        a.outD[gq] = D;
                        r_min[0] = fmin(r_min[0], (double)D);
                    }
                }
            }
        }
        __syncthreads();
        // (c) current, increment and outputs at plane kc = kk - 2
        const int kc = kk - 2;
        if (kc >= k0 && kc < kend) {
            const int i = i0 + tx, j = j0 + ty;
            if (i < p.nx && j < p.ny) {
                T Bc[3], Jv[3];
#pragma unroll
                for (int l = 0; l < 3; l++) Bc[l] = t.b(kc, l, j, i);
                if ((p.jOct || p.jQuint || p.jTri) && !a.jpass) {
                    // the octilateral / quintilateral current, computed after the J pass
                    const long long lj = (long long)i + (long long)p.nx * ((long long)j + (long long)p.ny * kc);
                    Jv[0] = a.outJ[3 * lj]; Jv[1] = a.outJ[3 * lj + 1]; Jv[2] = a.outJ[3 * lj + 2];
                } else if (p.jClassic) {
                    j_classic<T>(p, t, a.B0, i, j, kc, Jv);
                } else {
                    T xn[6][3], bn[6][3];
                    const int di[6] = {-1, 1, 0, 0, 0, 0}, dj[6] = {0, 0, -1, 1, 0, 0}, dk[6] = {0, 0, 0, 0, -1, 1};
#pragma unroll
                    for (int q = 0; q < 6; q++)
#pragma unroll
                        for (int l = 0; l < 3; l++) {
                            xn[q][l] = t.x(kc + dk[q], l, j + dj[q], i + di[q]);
                            bn[q][l] = t.b(kc + dk[q], l, j + dj[q], i + di[q]);
                        }
                    stokes<T>(xn, bn, Jv);
                }
                const long long lin = (long long)i + (long long)p.nx * ((long long)j + (long long)p.ny * kc);
                const long long klin = (long long)i + (long long)p.kpx * ((long long)j + (long long)p.ny * kc);
                const long long KC = p.kcs;
                if (MODE == MODE_STAGE) {
                    T kn[3];
                    T g[3] = {0, 0, 0};
                    if (PRESS) grad_p<T>(p, t, i, j, kc, t.b(kc, 3, j, i), g);
                    // inertia: the stage velocity u_n and its increment
                    T uc[3] = {0, 0, 0}, ku[3] = {0, 0, 0};
                    if (!p.inertia) {
                        cross3(Jv, Bc, kn);
                        if (p.jxbAver) {
                            // rungeKutta.cu:172-178, 357-443: J x B at the six face
                            // neighbours from this stage's J (inner) and B (ghosted),
                            // written by the J pass; the +z neighbour's B with the
                            // reference's plane stride (nx+1)(ny+1)
                            const T w6 = p.jxbW / (T)6;
                            const long long nx2 = p.nx + 2, ny2 = p.ny + 2;
#pragma unroll
                            for (int l = 0; l < 3; l++) kn[l] *= ((T)1 - p.jxbW);
#pragma unroll
                            for (int m = 0; m < 6; m++) {
                                bool in = false;
                                long long qj = 0, qb = 0;
                                if (m == 0) { in = i > 0; qj = lin - 1; qb = i + nx2 * ((j + 1) + ny2 * (long long)(kc + 1)); }
                                else if (m == 1) { in = i < p.nx - 1; qj = lin + 1; qb = (i + 2) + nx2 * ((j + 1) + ny2 * (long long)(kc + 1)); }
                                else if (m == 2) { in = j > 0; qj = lin - p.nx; qb = (i + 1) + nx2 * (j + ny2 * (long long)(kc + 1)); }
                                else if (m == 3) { in = j < p.ny - 1; qj = lin + p.nx; qb = (i + 1) + nx2 * ((j + 2) + ny2 * (long long)(kc + 1)); }
                                else if (m == 4) { in = kc > 0; qj = lin - (long long)p.nx * p.ny; qb = (i + 1) + nx2 * ((j + 1) + ny2 * (long long)kc); }
                                else { in = kc < p.nz - 1; qj = lin + (long long)p.nx * p.ny;
                                       qb = (i + 1) + nx2 * (j + 1) + (long long)(kc + 2) * (p.nx + 1) * (p.ny + 1); }
                                T c[3] = {0, 0, 0};
                                if (in) {
                                    const T jn[3] = {a.outJ[3 * qj], a.outJ[3 * qj + 1], a.outJ[3 * qj + 2]};
                                    const T bn[3] = {a.outB[3 * qb], a.outB[3 * qb + 1], a.outB[3 * qb + 2]};
                                    cross3(jn, bn, c);
                                }
#pragma unroll
                                for (int l = 0; l < 3; l++) kn[l] += c[l] * w6;
                            }
                        }
                        const T eps = p.ex[i] * p.ey[j] * p.ez[kc];
                        const T f = dtT * eps;
#pragma unroll
                        for (int l = 0; l < 3; l++) kn[l] *= f;
                        if (PRESS) {
#pragma unroll
                            for (int l = 0; l < 3; l++) kn[l] += -dtT * g[l];
                        }
                    } else {
                        // rungeKutta.cu:195-212: k_x = dt u, k_u = dt Delta (J x B)
                        // - dt nu u Delta - dt grad p (no epsilon profile)
                        const T* Un = (n == 0) ? a.U[cur] : a.US[(n - 1) & 1];
                        const T D = t.b(kc, 3, j, i);
                        cross3(Jv, Bc, ku);
#pragma unroll
                        for (int l = 0; l < 3; l++) {
                            uc[l] = Un[l * KC + klin];
                            kn[l] = dtT * uc[l];
                            ku[l] *= dtT * D;
                            ku[l] -= dtT * p.nu * uc[l] * D;
                            if (PRESS) ku[l] += -dtT * g[l];
                        }
                        if (!finite3d((double)ku[0], (double)ku[1], (double)ku[2])) bad = true;
                    }
                    if (!finite3d((double)kn[0], (double)kn[1], (double)kn[2])) bad = true;
                    T xa[3];
#pragma unroll
                    for (int l = 0; l < 3; l++) xa[l] = t.x(kc, l, j, i);
                    if (!LAST) {
                        // x_{n+1} = x_n + sum_{m<=n} (b[n+1][m] - b[n][m]) k_m  (rungeKutta.cu:216-227)
                        for (int m = 0; m < n; m++) {
                            const T* Km = a.K[m];
                            const T k0v = __ldg(&Km[klin]), k1v = __ldg(&Km[KC + klin]), k2v = __ldg(&Km[2 * KC + klin]);
                            const T w = p.db[n][m];
                            xa[0] += w * k0v;
                            xa[1] += w * k1v;
                            xa[2] += w * k2v;
                        }
                        const T w = p.db[n][n];
#pragma unroll
                        for (int l = 0; l < 3; l++) xa[l] += w * kn[l];
                        T* Kn = a.K[n];
                        Kn[klin] = kn[0];
                        Kn[KC + klin] = kn[1];
                        Kn[2 * KC + klin] = kn[2];
                        store_pos<T>(p, a.XS[n & 1], i, j, kc, xa);
                        if (p.inertia) {
                            // u_{n+1} = u_n + sum_{m<=n} (b[n+1][m] - b[n][m]) k_u,m
                            T ua[3] = {uc[0], uc[1], uc[2]};
                            for (int m = 0; m < n; m++) {
                                const T w = p.db[n][m];
#pragma unroll
                                for (int l = 0; l < 3; l++) ua[l] += w * __ldg(&a.KU[m][l * KC + klin]);
                            }
#pragma unroll
                            for (int l = 0; l < 3; l++) {
                                ua[l] += p.db[n][n] * ku[l];
                                a.KU[n][l * KC + klin] = ku[l];
                                a.US[n & 1][l * KC + klin] = ua[l];
                            }
                        }
                    } else {
                        // stage 5: x_6, then x_new, x* and the error norm (rungeKutta.cu:251-339)
                        T km[6][3];
#pragma unroll
                        for (int m = 0; m < 5; m++) {
                            km[m][0] = __ldg(&a.K[m][klin]);
                            km[m][1] = __ldg(&a.K[m][KC + klin]);
                            km[m][2] = __ldg(&a.K[m][2 * KC + klin]);
                        }
#pragma unroll
                        for (int l = 0; l < 3; l++) km[5][l] = kn[l];
#pragma unroll
                        for (int m = 0; m < 6; m++)
#pragma unroll
                            for (int l = 0; l < 3; l++) xa[l] += p.db[5][m] * km[m][l];
                        T xnew[3], xst[3];
#pragma unroll
                        for (int l = 0; l < 3; l++) {
                            xnew[l] = xa[l];
                            xst[l] = xa[l];
                            double dl = 0;
                            if (l < 2 || p.zUpdate) {
                                if (p.errMode == 0) {
#pragma unroll
                                    for (int m = 0; m < 6; m++) {
                                        xnew[l] += p.c[m] * km[m][l];
                                        xst[l] += p.cst[m] * km[m][l];
                                    }
                                    dl = (double)fabs(xnew[l] - xst[l]);
                                } else {
                                    double e = 0;
#pragma unroll
                                    for (int m = 0; m < 6; m++) {
                                        xnew[l] += p.c[m] * km[m][l];
                                        e += p.cmc[m] * (double)km[m][l];
                                    }
                                    dl = fabs(e);
                                }
                            }
                            if (dl > dmax) dmax = dl;     // NaN never wins (maths.cu:144-153)
                        }
                        store_pos<T>(p, a.X[cur], i, j, kc, xa);
                        store_pos<T>(p, a.X[cur ^ 1], i, j, kc, xnew);
                        if (p.inertia) {
                            // u_6 and u_new = u_6 + sum c k_u (rungeKutta.cu:311-322)
#pragma unroll
                            for (int l = 0; l < 3; l++) {
                                T kum[6];
#pragma unroll
                                for (int m = 0; m < 5; m++) kum[m] = __ldg(&a.KU[m][l * KC + klin]);
                                kum[5] = ku[l];
                                T u6 = uc[l];
#pragma unroll
                                for (int m = 0; m < 6; m++) u6 += p.db[5][m] * kum[m];
                                T un = u6;
#pragma unroll
                                for (int m = 0; m < 6; m++) un += p.c[m] * kum[m];
                                a.U[cur][l * KC + klin] = u6;
                                a.U[cur ^ 1][l * KC + klin] = un;
                            }
                        }
                    }
                } else {
                    // refresh and reductions (diagnostics.cu:12-134)
                    const T D = t.b(kc, 3, j, i);
                    const long long gq = (long long)(i + 1) + (long long)(p.nx + 2) * ((long long)(j + 1) + (long long)(p.ny + 2) * (kc + 1));
                    a.outB[3 * gq + 0] = Bc[0];
                    a.outB[3 * gq + 1] = Bc[1];
                    a.outB[3 * gq + 2] = Bc[2];
                    a.outD[gq] = D;
                    a.outJ[3 * lin + 0] = Jv[0];
                    a.outJ[3 * lin + 1] = Jv[1];
                    a.outJ[3 * lin + 2] = Jv[2];
                    T jxb[3];
                    cross3(Jv, Bc, jxb);
                    const T b2 = Bc[0] * Bc[0] + Bc[1] * Bc[1] + Bc[2] * Bc[2];
                    const T q1 = sqrt(jxb[0] * jxb[0] + jxb[1] * jxb[1] + jxb[2] * jxb[2]) / b2;
                    const double bx = Bc[0], by = Bc[1], bz = Bc[2], jx = Jv[0], jy = Jv[1], jz = Jv[2];
                    const double bnm = sqrt(bx * bx + by * by + bz * bz), jnm = sqrt(jx * jx + jy * jy + jz * jz);
                    const double cx = jy * bz - jz * by, cy = jz * bx - jx * bz, cz = jx * by - jy * bx;
                    const double cn = sqrt(cx * cx + cy * cy + cz * cz);
                    r_sum[0] += cn;
                    r_sum[1] += jnm * bnm;
                    if (jnm * bnm > 0) r_sum[2] += cn / (jnm * bnm);
                    const int bound = (i == 0) + (j == 0) + (kc == 0) + (i == p.nx - 1) + (j == p.ny - 1) + (kc == p.nz - 1);
                    r_sum[3] += (double)b2 * (double)D / (double)(1 << bound);
                    r_sum[4] += bx * bx + by * by + (bz - 1.0) * (bz - 1.0);
                    if (p.wantXbAn) {
                        // distance to the analytically relaxed grid (maths.cu:332-377)
                        const double X = (double)(p.dx * (T)i + p.Ox), Y = (double)(p.dy * (T)j + p.Oy),
                                     Z = (double)(p.dz * (T)kc + p.Oz);
                        const double ph = exp(-(X * X + Y * Y) / (p.ar * p.ar) - Z * Z / (p.az * p.az)) * p.phi1;
                        const double sp = sin(ph), cp = cos(ph);
                        const double a0 = (double)t.x(kc, 0, j, i) - cp * X - sp * Y;
                        const double a1 = (double)t.x(kc, 1, j, i) + sp * X - cp * Y;
                        const double a2 = (double)t.x(kc, 2, j, i) - Z;
                        r_sum[5] += a0 * a0 + a1 * a1 + a2 * a2;
                    }
                    r_max[0] = fmax(r_max[0], (double)q1);
                    r_max[1] = fmax(r_max[1], bnm);
                    r_max[2] = fmax(r_max[2], jnm);
                    if (p.inertia) {
                        // kinetic energy sum |u|^2 Delta with the boundary weights
                        // (maths.cu:684-710) and max |u| (mag, maths.cu)
                        const T* Uc = a.U[cur];
                        const double u0 = Uc[klin], u1 = Uc[KC + klin], u2 = Uc[2 * KC + klin];
                        const T uu2 = (T)u0 * (T)u0 + (T)u1 * (T)u1 + (T)u2 * (T)u2;
                        r_sum[6] += (double)(uu2 * D) / (double)(1 << bound);
                        r_max[3] = fmax(r_max[3], sqrt(u0 * u0 + u1 * u1 + u2 * u2));
                    }
                    r_min[0] = fmin(r_min[0], (double)D);
                    // wedge products and convexity (maths.cu:497-643)
                    T wmin = 0;
                    double conv = 1.0;
#pragma unroll
                    for (int u = 0; u < 2; u++)
#pragma unroll
                        for (int v = 0; v < 2; v++)
#pragma unroll
                            for (int w = 0; w < 2; w++) {
                                T d1[3], d2[3], d3[3], cc[3];
#pragma unroll
                                for (int l = 0; l < 3; l++) {
                                    const T xc = t.x(kc, l, j, i);
                                    d1[l] = t.x(kc, l, j, i + 2 * u - 1) - xc;
                                    d2[l] = t.x(kc, l, j + 2 * v - 1, i) - xc;
                                    d3[l] = t.x(kc + 2 * w - 1, l, j, i) - xc;
                                }
                                cross3(d1, d2, cc);
                                T wc = cc[0] * d3[0] + cc[1] * d3[1] + cc[2] * d3[2];
                                const int s = 2 * (u + v + w);
                                if ((wc < 0) && (s == 2 || s == 6)) conv = -1.0;
                                if ((wc > 0) && (s == 0 || s == 4)) conv = -1.0;
                                if (s == 0) wmin = -wc;
                                if (s == 0 || s == 4) wc = -wc;
                                if (wc < wmin) wmin = wc;
                            }
                    r_min[1] = fmin(r_min[1], (double)wmin);
                    r_min[2] = fmin(r_min[2], conv);
                }
            }
        }
    }

    if (MODE == MODE_STAGE) {
        if (bad) atomicOr(&st->status, (unsigned)GM_ST_NAN);
        if (LAST) {
            // CTA max of the error norm, then one atomic per CTA
            __shared__ double wmax[8];
            for (int o = 16; o > 0; o >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
            if (tx == 0) wmax[ty] = dmax;
            __syncthreads();
            if (tid == 0) {
                double m = 0;
                for (int w = 0; w < TY; w++) m = fmax(m, wmax[w]);
                if (m > 0) atomicMax(&st->maxDeltaBits, (unsigned long long)__double_as_longlong(m));
            }
        }
    } else {
        // deterministic CTA partials: fixed-order reduction through shared memory
        __syncthreads();
        double* red = reinterpret_cast<double*>(smraw);
        const double vals[R_COUNT] = {r_sum[0], r_sum[1], r_sum[2], r_sum[3], r_sum[4], r_sum[5], r_sum[6],
                                      r_max[0], r_max[1], r_max[2], r_max[3], r_min[0], r_min[1], r_min[2]};
        for (int r = 0; r < R_COUNT; r++) red[r * nthr + tid] = vals[r];
        __syncthreads();
        if (tid < R_COUNT) {
            const int r = tid;
            double acc = red[r * nthr];
            for (int q = 1; q < nthr; q++) {
                const double v = red[r * nthr + q];
                if (r <= R_LAST_SUM) acc += v;
                else if (r <= R_LAST_MAX) acc = fmax(acc, v);
                else acc = fmin(acc, v);
            }
            const int blin = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
            a.part[(long long)blin * R_COUNT + r] = acc;
        }
    }
}

// Accept/reject and the dt rule, src/main.cu:321-383, on the device.
template <typename T>
__device__ __forceinline__ void control_one(const KP<T>& p, DevState* st, double* log) {
    if (st->done) return;
    if (st->status & (GM_ST_TIMEOUT | GM_ST_ALIGN)) {
        // a stage of this step gave up a bounded wait or failed its alignment
        // check: its outputs are incomplete, so the step is neither accepted
        // nor used to adapt dt, and the run stops
        st->maxDeltaBits = 0ull;
        st->nAttempted++;
        st->nRejected++;
        st->lastAccepted = 0;
        st->event = 0;
        st->done = 1;
        st->status |= GM_ST_DONE;
        return;
    }
    const double md = __longlong_as_double((long long)st->maxDeltaBits);
    st->maxDeltaBits = 0ull;
    st->maxDelta = md;
    const int att = st->nAttempted++;
    const bool acc = md < p.maxError;
    const double dtOld = st->dt;
    st->lastAccepted = acc ? 1 : 0;
    if (acc) {
        st->t = p.refDt ? (double)((T)st->t + (T)st->dt) : st->t + st->dt;
        st->cur ^= 1;
        st->timeIndex++;
    } else {
        st->nRejected++;
    }
    if (md > 0) {
        const double ex = p.refDt ? (double)(T)0.2 : 0.2;
        const double nd = st->dt * pow(0.9 * p.maxError / md, ex);
        st->dt = p.refDt ? (double)(T)nd : nd;
    }
    st->dtUsed = dtOld;
    // output due after this step (main.cu:355-377): the time-series cadence
    // uses the loop index of the step, the dump triggers t and the adapted dt
    // in REAL, the last step is the one that reaches the target
    int ev = 0;
    if (acc) {
        const int ti = st->timeIndex - 1;
        if (p.nTs > 0 && ti % p.nTs == 0) ev |= GM_EV_TS;
        const T tt = (T)st->t, dd = (T)st->dt;
        if (ceil((T)(tt - dd) / p.dtDump) != ceil(tt / p.dtDump)) ev |= GM_EV_DUMP;
        if (ceil((T)(tt - dd) / p.dtSave) != ceil(tt / p.dtSave)) ev |= GM_EV_SAVE;
        if (st->timeIndex >= st->target) ev |= GM_EV_LAST;
    }
    st->event = ev;
    if (log && att < st->logCap) {
        log[3 * att] = md;
        log[3 * att + 1] = st->dt;
        log[3 * att + 2] = acc ? 1.0 : 0.0;
    }
    if (st->status & (GM_ST_NAN | GM_ST_TIMEOUT | GM_ST_ALIGN)) st->done = 1;
    if (!(st->dt > p.dtMin)) {
        st->status |= GM_ST_DTMIN;
        st->done = 1;
    }
    if (st->timeIndex >= st->target) st->done = 1;
    if (st->eventsOn && ev) {
        st->done = 1;
        st->status |= GM_ST_EVENT;
    }
    if (st->done) st->status |= GM_ST_DONE;
}

template <typename T>
__global__ void k_control(const __grid_constant__ KP<T> p, DevState* st, double* log) {
    control_one<T>(p, st, log);
}

// The controllers of a batch of cases, one thread each; also re-arms the six
// work counters of the batched stage launches for the next step.
template <typename T>
__global__ void k_control_batch(const StageArgsTMA<T>* __restrict__ cases, int ncases, int* __restrict__ counters) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < 6) counters[c] = 0;
    if (c < ncases) control_one<T>(cases[c].a.p, cases[c].a.st, cases[c].a.log);
}

// Fixed-order reduction of the CTA partials.
template <typename T>
__global__ void k_finalize(const double* __restrict__ part, int nparts, double* out) {
    __shared__ double red[R_COUNT][256];
    const int tid = threadIdx.x;
    for (int r = 0; r < R_COUNT; r++) {
        double acc = r <= R_LAST_SUM ? 0.0 : (r <= R_LAST_MAX ? 0.0 : DBL_MAX);
        if (r == R_MIN_CONVEX) acc = 1.0;
        for (int q = tid; q < nparts; q += blockDim.x) {
            const double v = part[(long long)q * R_COUNT + r];
            if (r <= R_LAST_SUM) acc += v;
            else if (r <= R_LAST_MAX) acc = fmax(acc, v);
            else acc = fmin(acc, v);
        }
        red[r][tid] = acc;
    }
    __syncthreads();
    if (tid < R_COUNT) {
        const int r = tid;
        double acc = red[r][0];
        for (int q = 1; q < (int)blockDim.x; q++) {
            const double v = red[r][q];
            if (r <= R_LAST_SUM) acc += v;
            else if (r <= R_LAST_MAX) acc = fmax(acc, v);
            else acc = fmin(acc, v);
        }
        out[r] = acc;
    }
}

template <typename T>
__global__ void k_unpack(const KP<T> p, const T* __restrict__ aos, T* __restrict__ soa) {
    const long long NG = (long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < NG; q += (long long)gridDim.x * blockDim.x) {
        const int gi = (int)(q % (p.nx + 2));
        const long long r = q / (p.nx + 2);
        const int gj = (int)(r % (p.ny + 2));
        const int gk = (int)(r / (p.ny + 2));
        const long long g = gidx(p.px, p.py, gi - 1, gj - 1, gk - 1);
        soa[g] = aos[3 * q];
        soa[p.cs + g] = aos[3 * q + 1];
        soa[2 * p.cs + g] = aos[3 * q + 2];
    }
}

// Depth-2 periodic images of the inner points (the depth-1 ghost layer keeps
// the values the caller supplied, as the reference's first stage sees them).
template <typename T>
__global__ void k_images(const KP<T> p, T* __restrict__ soa) {
    const long long NP = (long long)(p.nx + 4) * (p.ny + 4) * (p.nz + 4);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < NP; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % (p.nx + 4)) - 2;
        const long long r = q / (p.nx + 4);
        const int j = (int)(r % (p.ny + 4)) - 2;
        const int k = (int)(r / (p.ny + 4)) - 2;
        const bool xo = i < 0 || i >= p.nx, yo = j < 0 || j >= p.ny, zo = k < 0 || k >= p.nz;
        if (!(xo || yo || zo)) continue;
        if ((xo && !p.xPeri) || (yo && !p.yPeri) || (zo && !p.zPeri)) continue;
        const bool depth2 = (i == -2 || i == p.nx + 1) || (j == -2 || j == p.ny + 1) || (k == -2 || k == p.nz + 1);
        if (!depth2) continue;
        const int wi = xo ? (i < 0 ? i + p.nx : i - p.nx) : i;
        const int wj = yo ? (j < 0 ? j + p.ny : j - p.ny) : j;
        const int wk = zo ? (k < 0 ? k + p.nz : k - p.nz) : k;
        const long long gs = gidx(p.px, p.py, wi, wj, wk), gd = gidx(p.px, p.py, i, j, k);
        T v0 = soa[gs], v1 = soa[p.cs + gs], v2 = soa[2 * p.cs + gs];
        if (xo) v0 = i < 0 ? (v0 - p.Lx) - p.dx : (v0 + p.Lx) + p.dx;
        if (yo) v1 = j < 0 ? (v1 - p.Ly) - p.dy : (v1 + p.Ly) + p.dy;
        if (zo) v2 = k < 0 ? (v2 - p.Lz) - p.dz : (v2 + p.Lz) + p.dz;
        soa[gd] = v0;
        soa[p.cs + gd] = v1;
        soa[2 * p.cs + gd] = v2;
    }
}

// B0 scaled for the algebraic B formula: (4 dy dz B0x, 4 dx dz B0y, 4 dx dy B0z)
// The positions the line-tied z ghost planes' B formula uses on an initially
// distorted grid (updateBbound's face-2 branch, src/boundaries.cu:63-107),
// for every inner column (i, j) of both z faces: the outer plane (x, y) and
// the four in-plane neighbours extrapolated at the reference's 16-wide block
// edges (x, y each), in the reference's order of operations, with addDist in
// device arithmetic as the reference evaluates it.  The ghost planes are fixed,
// so this runs once per upload.  tab[10 ((side ny + j) nx + i) + q].
template <typename T>
__global__ void k_shear_table(const KP<T> p, const T* __restrict__ X, T* __restrict__ tab) {
    const long long n = 2ll * p.nx * p.ny;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % p.nx), j = (int)((q / p.nx) % p.ny), side = (int)(q / ((long long)p.nx * p.ny));
        const int k = side ? p.nz : -1;
        T X1[3];
        for (int l = 0; l < 3; l++)
            X1[l] = X[l * p.cs + (i + 2) + (long long)p.px * ((j + 2) + (long long)p.py * (k + 2))];
        const T sg = (T)(2 * side - 1);
        const T zs = p.dz * sg + p.Oz + p.Lz * (T)side;
        const T zo = (T)2 * p.dz * sg + p.Oz + p.Lz * (T)side;
        T* t = tab + 10 * q;
        for (int l = 0; l < 2; l++) t[l] = X1[l] - add_dist(p, i, j, X1[2], l) + add_dist(p, i, j, zo, l);
        t[2] = X1[0] - p.dx - add_dist(p, i, j, zs, 0) + add_dist(p, i - 1, j, zs, 0);
        t[3] = X1[1] - add_dist(p, i, j, zs, 1) + add_dist(p, i - 1, j, zs, 1);
        t[4] = X1[0] + p.dx - add_dist(p, i, j, zs, 0) + add_dist(p, i + 1, j, zs, 0);
        t[5] = X1[1] - add_dist(p, i, j, zs, 1) + add_dist(p, i + 1, j, zs, 1);
        t[6] = X1[0] - add_dist(p, i, j, zs, 0) + add_dist(p, i, j - 1, zs, 0);
        t[7] = X1[1] - p.dy - add_dist(p, i, j, zs, 1) + add_dist(p, i, j - 1, zs, 1);
        t[8] = X1[0] - add_dist(p, i, j, zs, 0) + add_dist(p, i, j + 1, zs, 0);
        t[9] = X1[1] + p.dy - add_dist(p, i, j, zs, 1) + add_dist(p, i, j + 1, zs, 1);
    }
}

template <typename T>
__global__ void k_scale_b0(const KP<T> p, const T* __restrict__ B0, T* __restrict__ B0s) {
    const T w0 = 4 * p.dy * p.dz, w1 = 4 * p.dx * p.dz, w2 = 4 * p.dx * p.dy;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < p.cs; q += (long long)gridDim.x * blockDim.x) {
        B0s[q] = B0[q] * w0;
        B0s[p.cs + q] = B0[p.cs + q] * w1;
        B0s[2 * p.cs + q] = B0[2 * p.cs + q] * w2;
    }
}

template <typename T>
__global__ void k_pack(const KP<T> p, const T* __restrict__ soa, T* __restrict__ aos) {
    const long long NG = (long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < NG; q += (long long)gridDim.x * blockDim.x) {
        const int gi = (int)(q % (p.nx + 2));
        const long long r = q / (p.nx + 2);
        const int gj = (int)(r % (p.ny + 2));
        const int gk = (int)(r / (p.ny + 2));
        const long long g = gidx(p.px, p.py, gi - 1, gj - 1, gk - 1);
        aos[3 * q] = soa[g];
        aos[3 * q + 1] = soa[p.cs + g];
        aos[3 * q + 2] = soa[2 * p.cs + g];
    }
}

// k_m from the pitched SoA layout to the reference kk layout (inner AoS).
template <typename T>
__global__ void k_pack_k(const KP<T> p, const T* __restrict__ k, T* __restrict__ aos) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < p.N; q += (long long)gridDim.x * blockDim.x) {
        const long long i = q % p.nx, r = q / p.nx;
        const long long g = i + (long long)p.kpx * r;
        aos[3 * q] = k[g];
        aos[3 * q + 1] = k[p.kcs + g];
        aos[3 * q + 2] = k[2 * p.kcs + g];
    }
}

// Octilateral Stokes current (JStokes4th, src/current.cu:413-736) at every
// inner point, from the positions (padded SoA) and the ghosted B of the
// reference layout (as the J pass exports it, ghost edges included).  For
// each plane through the point, axes (u, v) = (x, y), (y, z), (z, x): the
// circulation of B around the eight neighbours (-1,-1) (0,-1) (1,-1) (1,0)
// (1,1) (0,1) (-1,1) (-1,0) and the area vector (1/2) of the corner cross
// products plus (1/4) of the inner diamond's; then the 3x3 solve.
template <typename T>
__global__ void k_j_oct(const __grid_constant__ StageArgs<T> a) {
    const KP<T>& p = a.p;
    // the stage's input grid (the step start for stage 0, chosen on the device)
    const T* __restrict__ X = a.n == 0 ? a.X[a.st->cur] : a.XS[(a.n - 1) & 1];
    const T* __restrict__ B = a.outB;
    T* __restrict__ J = a.outJ;
    const int ax[3][2] = {{0, 1}, {1, 2}, {2, 0}};
    const int ring[9][2] = {{0, 0}, {1, 0}, {2, 0}, {2, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}, {0, 0}};
    const int dia[5][2] = {{0, 1}, {1, 0}, {2, 1}, {1, 2}, {0, 1}};
    const long long nx2 = p.nx + 2, ny2 = p.ny + 2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < p.N; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % p.nx), j = (int)((q / p.nx) % p.ny), k = (int)(q / ((long long)p.nx * p.ny));
        auto xat = [&](const int o[3], int l) { return X[l * p.cs + gidx(p.px, p.py, i + o[0], j + o[1], k + o[2])]; };
        auto bat = [&](const int o[3], int l) {
            return B[3 * ((i + 1 + o[0]) + nx2 * ((j + 1 + o[1]) + ny2 * (long long)(k + 1 + o[2]))) + l];
        };
        T NA[3][3], II[3];
#pragma unroll
        for (int pl = 0; pl < 3; pl++) {
            T xr[9][3], br[9][3], dx[8][3], dd[4][3], c[4][3];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                int o[3] = {0, 0, 0};
                o[ax[pl][0]] = ring[e][0] - 1;
                o[ax[pl][1]] = ring[e][1] - 1;
#pragma unroll
                for (int l = 0; l < 3; l++) { xr[e][l] = xat(o, l); br[e][l] = bat(o, l); }
            }
#pragma unroll
            for (int l = 0; l < 3; l++) { xr[8][l] = xr[0][l]; br[8][l] = br[0][l]; }
            T I = 0;
#pragma unroll
            for (int l = 0; l < 3; l++) {
#pragma unroll
                for (int e = 0; e < 8; e++) dx[e][l] = xr[e + 1][l] - xr[e][l];
                I += (br[1][l] + br[0][l]) / 2 * dx[0][l] + (br[2][l] + br[1][l]) / 2 * dx[1][l] +
                     (br[3][l] + br[2][l]) / 2 * dx[2][l] + (br[4][l] + br[3][l]) / 2 * dx[3][l] +
                     (br[5][l] + br[4][l]) / 2 * dx[4][l] + (br[6][l] + br[5][l]) / 2 * dx[5][l] +
                     (br[7][l] + br[6][l]) / 2 * dx[6][l] + (br[8][l] + br[7][l]) / 2 * dx[7][l];
            }
#pragma unroll
            for (int e = 0; e < 4; e++) {
                int o0[3] = {0, 0, 0}, o1[3] = {0, 0, 0};
                o0[ax[pl][0]] = dia[e][0] - 1; o0[ax[pl][1]] = dia[e][1] - 1;
                o1[ax[pl][0]] = dia[e + 1][0] - 1; o1[ax[pl][1]] = dia[e + 1][1] - 1;
#pragma unroll
                for (int l = 0; l < 3; l++) dd[e][l] = xat(o1, l) - xat(o0, l);
            }
            II[pl] = I;
            cross3(dx[1], dx[2], c[0]);
            cross3(dx[3], dx[4], c[1]);
            cross3(dx[5], dx[6], c[2]);
            cross3(dx[7], dx[0], c[3]);
#pragma unroll
            for (int l = 0; l < 3; l++) NA[pl][l] = (c[0][l] + c[1][l] + c[2][l] + c[3][l]) / 2;
            cross3(dd[0], dd[1], c[0]);
            cross3(dd[1], dd[2], c[1]);
            cross3(dd[2], dd[3], c[2]);
            cross3(dd[3], dd[0], c[3]);
#pragma unroll
            for (int l = 0; l < 3; l++) NA[pl][l] += (c[0][l] + c[1][l] + c[2][l] + c[3][l]) / 4;
        }
        const T det = NA[0][0] * NA[1][1] * NA[2][2] + NA[0][1] * NA[1][2] * NA[2][0] + NA[0][2] * NA[1][0] * NA[2][1] -
                      NA[0][0] * NA[1][2] * NA[2][1] - NA[0][1] * NA[1][0] * NA[2][2] - NA[0][2] * NA[1][1] * NA[2][0];
        T N1[3][3];
        N1[0][0] = (NA[1][1] * NA[2][2] - NA[1][2] * NA[2][1]) / det;
        N1[0][1] = (NA[0][2] * NA[2][1] - NA[0][1] * NA[2][2]) / det;
        N1[0][2] = (NA[0][1] * NA[1][2] - NA[0][2] * NA[1][1]) / det;
        N1[1][0] = (NA[1][2] * NA[2][0] - NA[1][0] * NA[2][2]) / det;
        N1[1][1] = (NA[0][0] * NA[2][2] - NA[0][2] * NA[2][0]) / det;
        N1[1][2] = (NA[0][2] * NA[1][0] - NA[0][0] * NA[1][2]) / det;
        N1[2][0] = (NA[1][0] * NA[2][1] - NA[1][1] * NA[2][0]) / det;
        N1[2][1] = (NA[0][1] * NA[2][0] - NA[0][0] * NA[2][1]) / det;
        N1[2][2] = (NA[0][0] * NA[1][1] - NA[0][1] * NA[1][0]) / det;
#pragma unroll
        for (int l = 0; l < 3; l++) {
            T Jl = 0;
#pragma unroll
            for (int m = 0; m < 3; m++) Jl += N1[l][m] * II[m];
            J[3 * q + l] = Jl;
        }
    }
}

// Quintilateral Stokes current (JStokesQuint, src/current.cu:737-1199) at
// every inner point, from the positions and the exported ghosted B, as
// k_j_oct.  Per plane, axes (u, v, w) = (x, y, z), (y, z, x), (z, x, y) and
// P(a, b) the neighbour at in-plane offsets (a - 1, b - 1): the diamond through
// the face neighbours, with a corner triangle's two outer edges in place of one
// diamond edge where the orientation tests pick one.  The tests are the
// reference's as written: each later test reads the edge vectors the previous
// one stored, the third compares with 4 instead of 0, the first triangle's
// edges take the B averages of the other edge, and in the (y, z, x) and
// (z, x, y) planes the fourth triangle's second edge runs from P(1, 2), not
// P(0, 2), to P(0, 1) (src/current.cu:995-996, 1104-1105).
// With p.jTri, the triangular Stokes current (JStokesTri, src/current.cu:
// 1202-1681): the same tests, but a plane where they pick a triangle takes that
// triangle alone (its two outer edges and the reversed diamond edge) as the
// contour and half the outer edges' cross product as the area vector.  The
// reference adds that to an area vector it never set (src/current.cu:1420-
// 1424), and its compiled kernel returns NaN in J wherever a plane takes a
// triangle; the unset start is NaN here too, so the stage's NaN check stops
// the step there.
template <typename T>
__device__ __forceinline__ T quiet_nan() {
    if constexpr (sizeof(T) == 8) return __longlong_as_double(0x7ff8000000000000ll);
    else return __int_as_float(0x7fc00000);
}

template <typename T>
__global__ void k_j_quint(const __grid_constant__ StageArgs<T> a) {
    const KP<T>& p = a.p;
    const T* __restrict__ X = a.n == 0 ? a.X[a.st->cur] : a.XS[(a.n - 1) & 1];
    const T* __restrict__ Bg = a.outB;
    T* __restrict__ J = a.outJ;
    const int ax[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
    const long long nx2 = p.nx + 2, ny2 = p.ny + 2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < p.N; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % p.nx), j = (int)((q / p.nx) % p.ny), k = (int)(q / ((long long)p.nx * p.ny));
        T NA[3][3], II[3];
#pragma unroll
        for (int pl = 0; pl < 3; pl++) {
            T x[3][3][3], b[3][3][3], xwp[3], xwm[3];
#pragma unroll
            for (int aa = 0; aa < 3; aa++)
#pragma unroll
                for (int bb = 0; bb < 3; bb++) {
                    int o[3] = {0, 0, 0};
                    o[ax[pl][0]] = aa - 1; o[ax[pl][1]] = bb - 1;
                    const long long g = gidx(p.px, p.py, i + o[0], j + o[1], k + o[2]);
                    const long long gb = (i + 1 + o[0]) + nx2 * ((j + 1 + o[1]) + ny2 * (long long)(k + 1 + o[2]));
#pragma unroll
                    for (int l = 0; l < 3; l++) { x[aa][bb][l] = X[l * p.cs + g]; b[aa][bb][l] = Bg[3 * gb + l]; }
                }
            {
                int o[3] = {0, 0, 0};
                o[ax[pl][2]] = 1;
                const long long gp = gidx(p.px, p.py, i + o[0], j + o[1], k + o[2]);
                const long long gm = gidx(p.px, p.py, i - o[0], j - o[1], k - o[2]);
#pragma unroll
                for (int l = 0; l < 3; l++) { xwp[l] = X[l * p.cs + gp]; xwm[l] = X[l * p.cs + gm]; }
            }
            T dx1[3], dx2[3], dx3[3], dx4[3], dx5[3], dx6[3], c[3];
            int tri = 0;
#pragma unroll
            for (int l = 0; l < 3; l++) {
                dx1[l] = x[1][0][l] - x[1][1][l];
                dx2[l] = x[2][1][l] - x[1][1][l];
                dx3[l] = x[1][2][l] - x[1][1][l];
                dx4[l] = x[0][1][l] - x[1][1][l];
                dx5[l] = xwp[l] - x[1][1][l];
                dx6[l] = xwm[l] - x[1][1][l];
            }
            auto dot = [](const T* u, const T* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
            cross3(dx1, dx2, c);
            if (dot(c, dx5) < 0 || dot(c, dx6) > 0) {
#pragma unroll
                for (int l = 0; l < 3; l++) { dx5[l] = x[2][0][l] - x[1][0][l]; dx6[l] = x[2][1][l] - x[2][0][l]; }
                tri = 2;
            }
            if (tri != 0) {
                cross3(dx2, dx3, c);
                if (dot(c, dx5) < 0 || dot(c, dx6) > 0) {
#pragma unroll
                    for (int l = 0; l < 3; l++) { dx5[l] = x[2][2][l] - x[2][1][l]; dx6[l] = x[1][2][l] - x[2][2][l]; }
                    tri = 3;
                }
            }
            if (tri != 0) {
                cross3(dx3, dx4, c);
                if (dot(c, dx5) < 0 || dot(c, dx6) > 4) {
#pragma unroll
                    for (int l = 0; l < 3; l++) { dx5[l] = x[0][2][l] - x[1][2][l]; dx6[l] = x[0][1][l] - (pl == 0 ? x[0][2][l] : x[1][2][l]); }
                    tri = 4;
                }
            }
            cross3(dx4, dx1, c);
            if (tri != 0) {
                if (dot(c, dx5) < 0 || dot(c, dx6) > 0) {
#pragma unroll
                    for (int l = 0; l < 3; l++) { dx5[l] = x[1][0][l] - x[0][0][l]; dx6[l] = x[0][0][l] - x[0][1][l]; }
                    tri = 1;
                }
            }
            T I = 0;
#pragma unroll
            for (int l = 0; l < 3; l++) {
                dx1[l] = x[1][0][l] - x[0][1][l];
                dx2[l] = x[2][1][l] - x[1][0][l];
                dx3[l] = x[1][2][l] - x[2][1][l];
                dx4[l] = x[0][1][l] - x[1][2][l];
                if (p.jTri && tri != 0) {
                    // the triangle's closing edge: the diamond edge reversed
                    if (tri == 1) I -= (b[1][0][l] + b[0][1][l]) / 2 * dx1[l];
                    if (tri == 2) I -= (b[2][1][l] + b[1][0][l]) / 2 * dx2[l];
                    if (tri == 3) I -= (b[1][2][l] + b[2][1][l]) / 2 * dx3[l];
                    if (tri == 4) I -= (b[0][1][l] + b[1][2][l]) / 2 * dx4[l];
                } else {
                    if (tri != 1) I += (b[1][0][l] + b[0][1][l]) / 2 * dx1[l];
                    if (tri != 2) I += (b[2][1][l] + b[1][0][l]) / 2 * dx2[l];
                    if (tri != 3) I += (b[1][2][l] + b[2][1][l]) / 2 * dx3[l];
                    if (tri != 4) I += (b[0][1][l] + b[1][2][l]) / 2 * dx4[l];
                }
                if (tri == 1) I += (b[0][1][l] + b[0][0][l]) / 2 * dx5[l] + (b[1][0][l] + b[0][0][l]) / 2 * dx6[l];
                if (tri == 2) I += (b[1][0][l] + b[2][0][l]) / 2 * dx5[l] + (b[2][1][l] + b[2][0][l]) / 2 * dx6[l];
                if (tri == 3) I += (b[2][1][l] + b[2][2][l]) / 2 * dx5[l] + (b[1][2][l] + b[2][2][l]) / 2 * dx6[l];
                if (tri == 4) I += (b[1][2][l] + b[0][2][l]) / 2 * dx5[l] + (b[0][1][l] + b[0][2][l]) / 2 * dx6[l];
            }
            T c12[3], c23[3], c34[3], c41[3], c56[3] = {0, 0, 0};
            cross3(dx1, dx2, c12);
            cross3(dx2, dx3, c23);
            cross3(dx3, dx4, c34);
            cross3(dx4, dx1, c41);
            if (tri > 0) cross3(dx5, dx6, c56);
            II[pl] = I;
#pragma unroll
            for (int l = 0; l < 3; l++) {
                if (p.jTri && tri > 0) {
                    NA[pl][l] = quiet_nan<T>() + c56[l] / 2;
                } else {
                    NA[pl][l] = (c12[l] + c23[l] + c34[l] + c41[l]) / 4;
                    if (tri > 0) NA[pl][l] += c56[l] / 2;
                }
            }
        }
        const T det = NA[0][0] * NA[1][1] * NA[2][2] + NA[0][1] * NA[1][2] * NA[2][0] + NA[0][2] * NA[1][0] * NA[2][1] -
                      NA[0][0] * NA[1][2] * NA[2][1] - NA[0][1] * NA[1][0] * NA[2][2] - NA[0][2] * NA[1][1] * NA[2][0];
        const T det1 = (T)1 / det;
        T N1[3][3];
        N1[0][0] = (NA[1][1] * NA[2][2] - NA[1][2] * NA[2][1]) * det1;
        N1[0][1] = (NA[0][2] * NA[2][1] - NA[0][1] * NA[2][2]) * det1;
        N1[0][2] = (NA[0][1] * NA[1][2] - NA[0][2] * NA[1][1]) * det1;
        N1[1][0] = (NA[1][2] * NA[2][0] - NA[1][0] * NA[2][2]) * det1;
        N1[1][1] = (NA[0][0] * NA[2][2] - NA[0][2] * NA[2][0]) * det1;
        N1[1][2] = (NA[0][2] * NA[1][0] - NA[0][0] * NA[1][2]) * det1;
        N1[2][0] = (NA[1][0] * NA[2][1] - NA[1][1] * NA[2][0]) * det1;
        N1[2][1] = (NA[0][1] * NA[2][0] - NA[0][0] * NA[2][1]) * det1;
        N1[2][2] = (NA[0][0] * NA[1][1] - NA[0][1] * NA[1][0]) * det1;
#pragma unroll
        for (int l = 0; l < 3; l++) {
            T Jl = 0;
#pragma unroll
            for (int m = 0; m < 3; m++) Jl += N1[l][m] * II[m];
            J[3 * q + l] = Jl;
        }
    }
}

// Two k-layout arrays (x and velocity increments) into the reference's
// six-value kk record per inner point.
template <typename T>
__global__ void k_pack_k6(const KP<T> p, const T* __restrict__ kx, const T* __restrict__ ku, T* __restrict__ aos) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < p.N; q += (long long)gridDim.x * blockDim.x) {
        const long long i = q % p.nx, r = q / p.nx;
        const long long g = i + (long long)p.kpx * r;
#pragma unroll
        for (int l = 0; l < 3; l++) {
            aos[6 * q + l] = kx[l * p.kcs + g];
            aos[6 * q + 3 + l] = ku[l * p.kcs + g];
        }
    }
}

// Inner-point AoS (the reference's uu layout) into the pitched k layout.
template <typename T>
__global__ void k_unpack_k(const KP<T> p, const T* __restrict__ aos, T* __restrict__ k) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < p.N; q += (long long)gridDim.x * blockDim.x) {
        const long long i = q % p.nx, r = q / p.nx;
        const long long g = i + (long long)p.kpx * r;
        k[g] = aos[3 * q];
        k[p.kcs + g] = aos[3 * q + 1];
        k[2 * p.kcs + g] = aos[3 * q + 2];
    }
}

// Periodic ghost layers of the exported B (setPeriFace, boundaries.cu:450-488)
// and of detJac, one face pair per launch in the order z, y, x.
template <typename T>
__global__ void k_export_peri(const KP<T> p, T* __restrict__ B, T* __restrict__ D, int face) {
    const int nx2 = p.nx + 2, ny2 = p.ny + 2, nz2 = p.nz + 2;
    const int n1 = face == 0 ? ny2 : nx2;
    const int n2 = face == 2 ? ny2 : nz2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)n1 * n2; q += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(q % n1), b = (int)(q / n1);
        long long lo, hi, slo, shi;
        auto G = [&](int i, int j, int k) { return (long long)i + (long long)nx2 * ((long long)j + (long long)ny2 * k); };
        if (face == 2) { lo = G(a, b, 0); hi = G(a, b, p.nz + 1); slo = G(a, b, p.nz); shi = G(a, b, 1); }
        else if (face == 1) { lo = G(a, 0, b); hi = G(a, p.ny + 1, b); slo = G(a, p.ny, b); shi = G(a, 1, b); }
        else { lo = G(0, a, b); hi = G(p.nx + 1, a, b); slo = G(p.nx, a, b); shi = G(1, a, b); }
        for (int l = 0; l < 3; l++) {
            B[3 * lo + l] = B[3 * slo + l];
            B[3 * hi + l] = B[3 * shi + l];
        }
        D[lo] = D[slo];
        D[hi] = D[shi];
    }
}

// Grid-quality fields at the inner points of a padded grid, inner layout:
// the signed volume of the cell towards +x,+y,+z (dirCellVol,
// maths.cu:441-490), the convexity flag and the minimum of the 8 corner
// wedge products with the sign convention of gridConvexity / gridWedgeMin
// (maths.cu:494-643).
template <typename T>
__global__ void k_grid_fields(const KP<T> p, const T* __restrict__ X, T* __restrict__ cellVol,
                              T* __restrict__ convexity, T* __restrict__ wedgeMin) {
    const long long cs = p.cs;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < p.N; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % p.nx), j = (int)((q / p.nx) % p.ny), k = (int)(q / ((long long)p.nx * p.ny));
        auto at = [&](int ii, int jj, int kk, int l) {
            return X[l * cs + (ii + 2) + (long long)p.px * ((jj + 2) + (long long)p.py * (kk + 2))];
        };
        T xc[3];
        for (int l = 0; l < 3; l++) xc[l] = at(i, j, k, l);
        if (cellVol) {
            T d1[3], d2[3], d3[3], cc[3];
            for (int l = 0; l < 3; l++) {
                d1[l] = at(i + 1, j, k, l) - xc[l];
                d2[l] = at(i, j + 1, k, l) - xc[l];
                d3[l] = at(i, j, k + 1, l) - xc[l];
            }
            cross3(d1, d2, cc);
            cellVol[q] = cc[0] * d3[0] + cc[1] * d3[1] + cc[2] * d3[2];
        }
        T wmin = 0, conv = 1;
        for (int u = 0; u < 2; u++)
            for (int v = 0; v < 2; v++)
                for (int w = 0; w < 2; w++) {
                    T d1[3], d2[3], d3[3], cc[3];
                    for (int l = 0; l < 3; l++) {
                        d1[l] = at(i + 2 * u - 1, j, k, l) - xc[l];
                        d2[l] = at(i, j + 2 * v - 1, k, l) - xc[l];
                        d3[l] = at(i, j, k + 2 * w - 1, l) - xc[l];
                    }
                    cross3(d1, d2, cc);
                    T wc = cc[0] * d3[0] + cc[1] * d3[1] + cc[2] * d3[2];
                    const int s = 2 * (u + v + w);
                    if ((wc < 0) && (s == 2 || s == 6)) conv = -1;
                    if ((wc > 0) && (s == 0 || s == 4)) conv = -1;
                    if (s == 0) wmin = -wc;
                    if (s == 0 || s == 4) wc = -wc;
                    if (wc < wmin) wmin = wc;
                }
        if (convexity) convexity[q] = conv;
        if (wedgeMin) wedgeMin[q] = wmin;
    }
}

// eps* (maths.cu:203-290 with diagnostics.cu:32-47): along the central column
// i = nx/2, j = ny/2, a_k = J.B/B^2 and z_k = x_z; eps* is the largest
// sqrt(2) |(a_n - a_p)/(z_n - z_p)| over the pairs with z_n != z_p, in REAL;
// NaN values never win (maths.cu:144-153).  One CTA.
template <typename T>
__global__ void k_eps_star(const KP<T> p, const T* __restrict__ B, const T* __restrict__ J, const T* __restrict__ X,
                           T* __restrict__ sc, double* __restrict__ out) {
    const int i = p.nx / 2, j = p.ny / 2, nz = p.nz;
    T* a = sc;
    T* z = sc + nz;
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        const long long g = (long long)(i + 1) + (long long)(p.nx + 2) * ((j + 1) + (long long)(p.ny + 2) * (k + 1));
        const long long l = (long long)i + (long long)p.nx * (j + (long long)p.ny * k);
        const T b0 = B[3 * g], b1 = B[3 * g + 1], b2 = B[3 * g + 2];
        const T j0 = J[3 * l], j1 = J[3 * l + 1], j2 = J[3 * l + 2];
        a[k] = (j0 * b0 + j1 * b1 + j2 * b2) / (b0 * b0 + b1 * b1 + b2 * b2);
        z[k] = X[2 * p.cs + (i + 2) + (long long)p.px * ((j + 2) + (long long)p.py * (k + 2))];
    }
    __syncthreads();
    T m = 0;    // every value is >= 0, and the pairs n == p give 0
    for (int q = threadIdx.x; q < nz * nz; q += blockDim.x) {
        const int pp = q / nz, n = q % nz;
        if (z[n] != z[pp]) {
            const T v = (T)(1.414213562373095 * (double)fabs((a[n] - a[pp]) / (z[n] - z[pp])));
            if (v > m) m = v;
        }
    }
    __shared__ double red[256];
    red[threadIdx.x] = (double)m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// ---- host launchers ---------------------------------------------------------

template <typename T>
size_t stage_smem_bytes(int TY, int mode, int pressure) {
    (void)pressure;
    const int NB = 4;
    size_t b = sizeof(T) * ((size_t)XRING * 3 * (TY + 4) * (TX + 4) + (size_t)BRING * NB * (TY + 2) * (TX + 2));
    if (mode == MODE_DIAG) b = b > (size_t)R_COUNT * TX * TY * sizeof(double) ? b : (size_t)R_COUNT * TX * TY * sizeof(double);
    return b;
}

template <typename T, bool PRESS, int MODE, bool LAST>
static cudaError_t launch_one(const StageArgs<T>& a, dim3 grid, dim3 block, size_t smem, cudaStream_t s) {
    k_stage<T, PRESS, MODE, LAST><<<grid, block, smem, s>>>(a);
    return cudaGetLastError();
}

// Resident CTAs per SM of the stage kernel for a tile height and smem size.
template <typename T>
int stage_occupancy(int TY, int pressure, size_t smem) {
    int nb = 0;
    cudaError_t e = pressure
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_stage<T, true, MODE_STAGE, false>, TX * TY, smem)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_stage<T, false, MODE_STAGE, false>, TX * TY, smem);
    return e == cudaSuccess && nb > 0 ? nb : 1;
}

// Opt every stage-kernel variant in to large dynamic shared memory (once per
// device, before any launch or stream capture).
template <typename T>
cudaError_t prepare_kernels() {
    const int lim = 200 * 1024;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_stage<T, false, MODE_STAGE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim))) return e;
    if ((e = cudaFuncSetAttribute(k_stage<T, false, MODE_STAGE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim))) return e;
    if ((e = cudaFuncSetAttribute(k_stage<T, true, MODE_STAGE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim))) return e;
    if ((e = cudaFuncSetAttribute(k_stage<T, true, MODE_STAGE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim))) return e;
    if ((e = cudaFuncSetAttribute(k_stage<T, false, MODE_DIAG, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim))) return e;
    return cudaFuncSetAttribute(k_stage<T, true, MODE_DIAG, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
}

template <typename T>
cudaError_t launch_stage(const StageArgs<T>& a, int mode, int pressure, dim3 grid, dim3 block, size_t smem,
                         cudaStream_t s) {
    if (mode == MODE_DIAG)
        return pressure ? launch_one<T, true, MODE_DIAG, false>(a, grid, block, smem, s)
                        : launch_one<T, false, MODE_DIAG, false>(a, grid, block, smem, s);
    const bool last = a.n == 5;
    if (pressure)
        return last ? launch_one<T, true, MODE_STAGE, true>(a, grid, block, smem, s)
                    : launch_one<T, true, MODE_STAGE, false>(a, grid, block, smem, s);
    return last ? launch_one<T, false, MODE_STAGE, true>(a, grid, block, smem, s)
                : launch_one<T, false, MODE_STAGE, false>(a, grid, block, smem, s);
}

template <typename T>
cudaError_t launch_control(const KP<T>& p, DevState* st, double* log, cudaStream_t s) {
    k_control<T><<<1, 1, 0, s>>>(p, st, log);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_control_batch(const StageArgsTMA<T>* cases, int ncases, int* counters, cudaStream_t s) {
    const int n = ncases > 6 ? ncases : 6;
    k_control_batch<T><<<(n + 127) / 128, 128, 0, s>>>(cases, ncases, counters);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_finalize(const double* part, int nparts, double* out, cudaStream_t s) {
    k_finalize<T><<<1, 256, 0, s>>>(part, nparts, out);
    return cudaGetLastError();
}

static inline unsigned nblk(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

template <typename T>
cudaError_t launch_unpack(const KP<T>& p, const T* aos, T* soa, cudaStream_t s) {
    k_unpack<T><<<nblk((long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2)), 256, 0, s>>>(p, aos, soa);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_shear_table(const KP<T>& p, const T* X, T* tab, cudaStream_t s) {
    k_shear_table<T><<<nblk(2ll * p.nx * p.ny), 256, 0, s>>>(p, X, tab);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_scale_b0(const KP<T>& p, const T* B0, T* B0s, cudaStream_t s) {
    k_scale_b0<T><<<nblk(p.cs), 256, 0, s>>>(p, B0, B0s);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_images(const KP<T>& p, T* soa, cudaStream_t s) {
    k_images<T><<<nblk((long long)(p.nx + 4) * (p.ny + 4) * (p.nz + 4)), 256, 0, s>>>(p, soa);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pack(const KP<T>& p, const T* soa, T* aos, cudaStream_t s) {
    k_pack<T><<<nblk((long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2)), 256, 0, s>>>(p, soa, aos);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pack_k(const KP<T>& p, const T* k, T* aos, cudaStream_t s) {
    k_pack_k<T><<<nblk(p.N), 256, 0, s>>>(p, k, aos);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_j_oct(const StageArgs<T>& a, cudaStream_t s) {
    k_j_oct<T><<<nblk(a.p.N), 128, 0, s>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_j_quint(const StageArgs<T>& a, cudaStream_t s) {
    k_j_quint<T><<<nblk(a.p.N), 128, 0, s>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pack_k6(const KP<T>& p, const T* kx, const T* ku, T* aos, cudaStream_t s) {
    k_pack_k6<T><<<nblk(p.N), 256, 0, s>>>(p, kx, ku, aos);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_unpack_k(const KP<T>& p, const T* aos, T* k, cudaStream_t s) {
    k_unpack_k<T><<<nblk(p.N), 256, 0, s>>>(p, aos, k);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_export_ghosts(const KP<T>& p, T* outB, T* outD, cudaStream_t s) {
    const int nx2 = p.nx + 2, ny2 = p.ny + 2, nz2 = p.nz + 2;
    if (p.zPeri) k_export_peri<T><<<nblk((long long)nx2 * ny2), 256, 0, s>>>(p, outB, outD, 2);
    if (p.yPeri) k_export_peri<T><<<nblk((long long)nx2 * nz2), 256, 0, s>>>(p, outB, outD, 1);
    if (p.xPeri) k_export_peri<T><<<nblk((long long)ny2 * nz2), 256, 0, s>>>(p, outB, outD, 0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_grid_fields(const KP<T>& p, const T* X, T* cellVol, T* convexity, T* wedgeMin, cudaStream_t s) {
    k_grid_fields<T><<<nblk(p.N), 256, 0, s>>>(p, X, cellVol, convexity, wedgeMin);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_eps_star(const KP<T>& p, const T* B, const T* J, const T* X, T* scratch, double* out,
                            cudaStream_t s) {
    k_eps_star<T><<<1, 256, 0, s>>>(p, B, J, X, scratch, out);
    return cudaGetLastError();
}

#define GMK_INSTANTIATE(T)                                                                                        \
    template cudaError_t launch_stage<T>(const StageArgs<T>&, int, int, dim3, dim3, size_t, cudaStream_t);       \
    template size_t stage_smem_bytes<T>(int, int, int);                                                           \
    template cudaError_t prepare_kernels<T>();                                                                    \
    template int stage_occupancy<T>(int, int, size_t);                                                            \
    template cudaError_t launch_control<T>(const KP<T>&, DevState*, double*, cudaStream_t);                       \
    template cudaError_t launch_control_batch<T>(const StageArgsTMA<T>*, int, int*, cudaStream_t);                \
    template cudaError_t launch_finalize<T>(const double*, int, double*, cudaStream_t);                           \
    template cudaError_t launch_unpack<T>(const KP<T>&, const T*, T*, cudaStream_t);                              \
    template cudaError_t launch_pack<T>(const KP<T>&, const T*, T*, cudaStream_t);                                \
    template cudaError_t launch_images<T>(const KP<T>&, T*, cudaStream_t);                                        \
    template cudaError_t launch_scale_b0<T>(const KP<T>&, const T*, T*, cudaStream_t);                            \
    template cudaError_t launch_shear_table<T>(const KP<T>&, const T*, T*, cudaStream_t);                         \
    template cudaError_t launch_pack_k<T>(const KP<T>&, const T*, T*, cudaStream_t);                              \
    template cudaError_t launch_pack_k6<T>(const KP<T>&, const T*, const T*, T*, cudaStream_t);                  \
    template cudaError_t launch_j_oct<T>(const StageArgs<T>&, cudaStream_t);                                    \
    template cudaError_t launch_j_quint<T>(const StageArgs<T>&, cudaStream_t);                                  \
    template cudaError_t launch_unpack_k<T>(const KP<T>&, const T*, T*, cudaStream_t);                          \
    template cudaError_t launch_export_ghosts<T>(const KP<T>&, T*, T*, cudaStream_t);                            \
    template cudaError_t launch_grid_fields<T>(const KP<T>&, const T*, T*, T*, T*, cudaStream_t);                 \
    template cudaError_t launch_eps_star<T>(const KP<T>&, const T*, const T*, const T*, T*, double*, cudaStream_t);

}  // namespace gmk
