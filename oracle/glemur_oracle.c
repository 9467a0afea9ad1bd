/*
 * glemur_oracle.c -- ORACLE: test infrastructure only.
 *
 * A plain-C CPU restatement of the reference's magneto-frictional relaxation
 * hot path (SimonCan/glemur, src/).  It is the checker for the CUDA library in
 * glemur_gb300/: only the tests, the smoke check and the CPU-baseline leg of
 * bench.py load it.  The product path never calls into it.
 *
 * Parity pinning: the outputs of this restatement are checked against the
 * reference's own CUDA kernels (compiled from the reference sources into a
 * cubin and driven by oracle/ref/ref_launcher.cpp) through the golden
 * fixtures under tests/golden/.
 *
 * Compiled twice: -DORC_BITS=64 (REAL = double, PRECISION=64 build of the
 * reference) and -DORC_BITS=32 (REAL = float).  Build with
 * -ffp-contract=off so results do not depend on the host's FMA contraction.
 * Where the reference promotes to double inside a REAL expression (the
 * literal "1." in B_JacB0, the epsilon profile, the dt rule's pow) the same
 * promotion is written out here.
 *
 * Array layout is the reference's: AoS, component fastest, one ghost layer.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/glemur.h"

#ifndef ORC_BITS
#define ORC_BITS 64
#endif
#if ORC_BITS == 32
typedef float R;
#define REXP expf
#define RSIN sinf
#define RSQRT sqrtf
#define RABS fabsf
#else
typedef double R;
#define REXP exp
#define RSIN sin
#define RSQRT sqrt
#define RABS fabs
#endif

#define PI_D 3.141592653589793

/* REAL copy of the run parameters (src/global.h:44-108). */
typedef struct {
    int nx, ny, nz;
    R Lx, Ly, Lz, Ox, Oy, Oz, dx, dy, dz, dx1, dy1, dz1;
    R ampl, phi1, phi2, ar, az;
    int nBlobs;
    R blobXc[10], blobYc[10], blobZc[10], blobZl[10], blobTwist[10], blobScale[10];
    int initDistCode;
    R initShearA, initShearB, initShearK;
    int nCycle;
    R dt0, dtMin, maxError;
    int zUpdate, pressure, epsilonProf;
    R beta;
    int xPeri, yPeri, zPeri;
    int nTs;
    int errMode;
    R p0Amp, p0Width;
    int jClassic;              /* jMethod = "Classic" (else "Stokes")            */
    int jOct;                  /* jMethod = "Stokes4th": octilateral contours    */
    int jQuint;                /* jMethod = "StokesQuint": quintilaterals        */
    int jTri;                  /* jMethod = "StokesTri": diamonds or triangles   */
    int inertia;               /* the velocity equation (rungeKutta.cu:195-212)  */
    R nu;                      /* velocity damping                               */
    int jxbAver;               /* neighbour-averaged Lorentz force               */
    R jxbAverWeight;
} P;

typedef struct orc_state {
    P p;
    size_t NG, N;              /* ghosted and inner point counts               */
    R *B0, *B, *xb, *xb_tmp, *xb_new, *J, *kk, *detJac, *gradP;
    R *uu, *uu_tmp, *uu_new;   /* velocity (inertia): inner points, AoS          */
    int nVar;                  /* variables per point in kk: 3, or 6 with inertia */
    R t, dt;
    int timeIndex;
    R b[7][6], c[6], cs[6];
    R maxDelta;
    int nAttempted;
} orc_state;

static void to_P(const gm_params* g, P* p) {
    int b;
    p->nx = g->nx; p->ny = g->ny; p->nz = g->nz;
    p->Lx = (R)g->Lx; p->Ly = (R)g->Ly; p->Lz = (R)g->Lz;
    p->Ox = (R)g->Ox; p->Oy = (R)g->Oy; p->Oz = (R)g->Oz;
    p->dx = (R)g->dx; p->dy = (R)g->dy; p->dz = (R)g->dz;
    p->dx1 = (R)g->dx1; p->dy1 = (R)g->dy1; p->dz1 = (R)g->dz1;
    p->ampl = (R)g->ampl; p->phi1 = (R)g->phi1; p->phi2 = (R)g->phi2;
    p->ar = (R)g->ar; p->az = (R)g->az;
    p->nBlobs = g->nBlobs;
    for (b = 0; b < 10; b++) {
        p->blobXc[b] = (R)g->blobXc[b]; p->blobYc[b] = (R)g->blobYc[b];
        p->blobZc[b] = (R)g->blobZc[b]; p->blobZl[b] = (R)g->blobZl[b];
        p->blobTwist[b] = (R)g->blobTwist[b]; p->blobScale[b] = (R)g->blobScale[b];
    }
    p->initDistCode = g->initDistCode;
    p->initShearA = (R)g->initShearA; p->initShearB = (R)g->initShearB;
    p->initShearK = (R)g->initShearK;
    p->nCycle = g->nCycle;
    p->dt0 = (R)g->dt0; p->dtMin = (R)g->dtMin; p->maxError = (R)g->maxError;
    p->zUpdate = g->zUpdate; p->pressure = g->pressure; p->epsilonProf = g->epsilonProf;
    p->beta = (R)g->beta;
    p->xPeri = g->xPeri; p->yPeri = g->yPeri; p->zPeri = g->zPeri;
    p->nTs = g->nTs > 0 ? g->nTs : 1;
    p->errMode = g->errMode;
    p->p0Amp = (R)g->p0Amp; p->p0Width = (R)g->p0Width;
    p->jClassic = strncmp(g->jMethod, "Classic ", 8) == 0;
    p->jOct = strncmp(g->jMethod, "Stokes4th ", 10) == 0;
    p->jQuint = strncmp(g->jMethod, "StokesQuint ", 12) == 0;
    p->jTri = strncmp(g->jMethod, "StokesTri ", 10) == 0;
    p->inertia = g->inertia != 0;
    p->nu = (R)g->nu;
    p->jxbAver = g->jxbAver != 0;
    p->jxbAverWeight = (R)g->jxbAverWeight;
}

/* ghosted (i, j, k in 0..n+1) and inner (0..n-1) linear point indices */
#define GI(p, i, j, k) ((size_t)(i) + (size_t)((p)->nx + 2) * ((size_t)(j) + (size_t)((p)->ny + 2) * (size_t)(k)))
#define II(p, i, j, k) ((size_t)(i) + (size_t)(p)->nx * ((size_t)(j) + (size_t)(p)->ny * (size_t)(k)))

/* Cash-Karp tableau, src/rungeKutta.cu:10-25 (double literals rounded to REAL). */
static void assign_coefficients(R b[7][6], R c[6], R cs[6]) {
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
    int n, m;
    for (n = 0; n < 7; n++)
        for (m = 0; m < 6; m++) b[n][m] = (R)bd[n][m];
    for (m = 0; m < 6; m++) { c[m] = (R)cd[m]; cs[m] = (R)csd[m]; }
}

static R det3(R j[3][3]) {
    return j[0][0] * j[1][1] * j[2][2] + j[0][1] * j[1][2] * j[2][0] + j[0][2] * j[1][0] * j[2][1] -
           j[0][0] * j[1][2] * j[2][1] - j[0][1] * j[1][0] * j[2][2] - j[0][2] * j[1][1] * j[2][0];
}

static void cross3(const R a[3], const R b[3], R c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static R dot3(const R a[3], const R b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* ------------------------------------------------------------------------ */
/* Initial state: src/init.cu:30-384 ("blobs", "homZ", "analytic"), grid    */
/* src/init.cu:224-226, periodic B0 copy src/boundaries.cu:492-528.         */
/* ------------------------------------------------------------------------ */

static void set_peri_field(const P* p, R* f) {
    int i, j, l;
    /* order z, y, x as src/boundaries.cu:496-527 */
    if (p->zPeri)
        for (i = 0; i < p->nx + 2; i++)
            for (j = 0; j < p->ny + 2; j++)
                for (l = 0; l < 3; l++) {
                    f[3 * GI(p, i, j, 0) + l] = f[3 * GI(p, i, j, p->nz) + l];
                    f[3 * GI(p, i, j, p->nz + 1) + l] = f[3 * GI(p, i, j, 1) + l];
                }
    if (p->yPeri)
        for (i = 0; i < p->nx + 2; i++)
            for (j = 0; j < p->nz + 2; j++)
                for (l = 0; l < 3; l++) {
                    f[3 * GI(p, i, 0, j) + l] = f[3 * GI(p, i, p->ny, j) + l];
                    f[3 * GI(p, i, p->ny + 1, j) + l] = f[3 * GI(p, i, 1, j) + l];
                }
    if (p->xPeri)
        for (i = 0; i < p->ny + 2; i++)
            for (j = 0; j < p->nz + 2; j++)
                for (l = 0; l < 3; l++) {
                    f[3 * GI(p, 0, i, j) + l] = f[3 * GI(p, p->nx, i, j) + l];
                    f[3 * GI(p, p->nx + 1, i, j) + l] = f[3 * GI(p, 1, i, j) + l];
                }
}

/* initDistortion, src/init.cu:386-420: the grid, ghosts included (B0 refers
 * to the undistorted grid).  "initShearX" shears y by a sine of x and then x
 * by a sine of the sheared y, both growing linearly in z, in double
 * arithmetic as PI is a double constant; "centerShift" moves y by a Gaussian
 * in x, with a constant (5.08...) that differs from addDist's (0.15366). */
static void init_distortion(const gm_params* g, const P* p, R* xb) {
    int i, j, k;
    const int shear = strncmp(g->initDist, "initShearX ", 11) == 0;
    const int shift = strncmp(g->initDist, "centerShift ", 12) == 0;
    if (!shear && !shift) return;
    for (k = 0; k < p->nz + 2; k++) {
        R z = p->dz * (R)(k - 1) + p->Oz;
        for (j = 0; j < p->ny + 2; j++) {
            R y = p->dy * (R)(j - 1) + p->Oy;
            for (i = 0; i < p->nx + 2; i++) {
                R x = p->dx * (R)(i - 1) + p->Ox;
                R* xp = &xb[3 * GI(p, i, j, k)];
                if (shear) {
                    R yy;
                    xp[1] = (R)(xp[1] - p->initShearA * sin(p->initShearK * 2 * PI_D * (x + p->Ox - p->dx / 2) /
                                                            (p->Lx + p->dx)) * z);
                    yy = xp[1];
                    xp[0] = (R)(xp[0] - p->initShearB * sin(p->initShearK * 2 * PI_D * (yy + p->Oy - p->dy / 2) /
                                                            (p->Ly + p->dy)) * z);
                }
                if (shift)
                    xp[1] = (R)(xp[1] + p->initShearA * REXP(-p->initShearK * x * x) * (1 - y * y) *
                                            (REXP(-1 * z + 1) - 5.0804508111226507));
            }
        }
    }
}

int orc_init_state(const gm_params* g, R* B0, R* xb) {
    P p;
    int i, j, k, b;
    int mode;
    to_P(g, &p);
    if (strncmp(g->bInit, "blobs ", 6) == 0) mode = 0;
    else if (strncmp(g->bInit, "homZ ", 5) == 0) mode = 1;
    else if (strncmp(g->bInit, "analytic ", 9) == 0) mode = 2;
    else return GM_EPARAM;
    if (strncmp(g->initDist, "none ", 5) != 0 && strncmp(g->initDist, "initShearX ", 11) != 0 &&
        strncmp(g->initDist, "centerShift ", 12) != 0)
        return GM_EPARAM;
    for (k = 0; k < p.nz + 2; k++) {
        R z = p.dz * (R)(k - 1) + p.Oz;
        for (j = 0; j < p.ny + 2; j++) {
            R y = p.dy * (R)(j - 1) + p.Oy;
            for (i = 0; i < p.nx + 2; i++) {
                R x = p.dx * (R)(i - 1) + p.Ox;
                R* Bp = &B0[3 * GI(&p, i, j, k)];
                R* xp = &xb[3 * GI(&p, i, j, k)];
                if (mode == 2) {
                    R e = REXP(-(x * x + y * y) / (p.ar * p.ar) - z * z / (p.az * p.az));
                    Bp[0] = 2 * p.ampl * z * e * p.phi1 / (p.az * p.az) * y;
                    Bp[1] = -2 * p.ampl * z * e * p.phi1 / (p.az * p.az) * x;
                    Bp[2] = p.ampl;
                } else if (mode == 1) {
                    Bp[0] = 0.; Bp[1] = 0.; Bp[2] = p.ampl;
                } else {
                    Bp[0] = 0.; Bp[1] = 0.; Bp[2] = 0.;
                    for (b = 0; b < p.nBlobs; b++) {
                        R e = REXP((-(x - p.blobXc[b]) * (x - p.blobXc[b]) - (y - p.blobYc[b]) * (y - p.blobYc[b])) /
                                       (p.blobScale[b] * p.blobScale[b]) -
                                   (z - p.blobZc[b]) * (z - p.blobZc[b]) / (p.blobZl[b] * p.blobZl[b]));
                        Bp[0] += 2 * p.ampl * p.blobTwist[b] / p.blobScale[b] * e * (-(y - p.blobYc[b]));
                        Bp[1] += 2 * p.ampl * p.blobTwist[b] / p.blobScale[b] * e * (x - p.blobXc[b]);
                    }
                    Bp[2] = p.ampl;
                }
                xp[0] = x; xp[1] = y; xp[2] = z;
            }
        }
    }
    init_distortion(g, &p, xb);
    /* src/main.cu:168-169.  setGridPeriHost (boundaries.cu:586-634) leaves the
     * in-bounds grid unchanged: its shifted-component statements sit outside
     * the inner loop (missing braces) and only touch indices past the plane
     * range, and the copied components are equal on the identity grid.  So the
     * effective initial grid is the identity grid, ghosts included. */
    set_peri_field(&p, B0);
    return GM_OK;
}

/* ------------------------------------------------------------------------ */
/* State handling                                                            */
/* ------------------------------------------------------------------------ */

void orc_destroy(orc_state* s);

orc_state* orc_create(const gm_params* g, const R* B0, const R* xb, double t, double dt) {
    orc_state* s = (orc_state*)calloc(1, sizeof(orc_state));
    if (!s) return NULL;
    to_P(g, &s->p);
    s->NG = (size_t)(g->nx + 2) * (g->ny + 2) * (g->nz + 2);
    s->N = (size_t)g->nx * g->ny * g->nz;
    s->B0 = (R*)calloc(3 * s->NG, sizeof(R));
    s->B = (R*)calloc(3 * s->NG, sizeof(R));
    s->xb = (R*)calloc(3 * s->NG, sizeof(R));
    s->xb_tmp = (R*)calloc(3 * s->NG, sizeof(R));
    s->xb_new = (R*)calloc(3 * s->NG, sizeof(R));
    s->J = (R*)calloc(3 * s->N, sizeof(R));
    s->nVar = g->inertia ? 6 : 3;
    s->kk = (R*)calloc(6 * (size_t)s->nVar * s->N, sizeof(R));
    s->detJac = (R*)calloc(s->NG, sizeof(R));
    s->gradP = (R*)calloc(3 * s->N, sizeof(R));
    /* uInit = "nil": zero velocity (memory.cu:33-35 allocates uu with malloc
     * and init.cu:362-364 leaves it unset; zero-filled here) */
    s->uu = (R*)calloc(3 * s->N, sizeof(R));
    s->uu_tmp = (R*)calloc(3 * s->N, sizeof(R));
    s->uu_new = (R*)calloc(3 * s->N, sizeof(R));
    if (!s->B0 || !s->B || !s->xb || !s->xb_tmp || !s->xb_new || !s->J || !s->kk || !s->detJac || !s->gradP ||
        !s->uu || !s->uu_tmp || !s->uu_new) {
        orc_destroy(s);
        return NULL;
    }
    memcpy(s->B0, B0, 3 * s->NG * sizeof(R));
    memcpy(s->B, B0, 3 * s->NG * sizeof(R));       /* main.cu:195 */
    memcpy(s->xb, xb, 3 * s->NG * sizeof(R));
    memcpy(s->xb_tmp, xb, 3 * s->NG * sizeof(R));   /* main.cu:202 */
    memcpy(s->xb_new, xb, 3 * s->NG * sizeof(R));   /* main.cu:209 */
    s->t = (R)t;
    s->dt = (R)dt;
    s->timeIndex = 0;
    assign_coefficients(s->b, s->c, s->cs);
    return s;
}

void orc_destroy(orc_state* s) {
    if (!s) return;
    free(s->B0); free(s->B); free(s->xb); free(s->xb_tmp); free(s->xb_new);
    free(s->J); free(s->kk); free(s->detJac); free(s->gradP);
    free(s->uu); free(s->uu_tmp); free(s->uu_new);
    free(s);
}

void orc_get(const orc_state* s, R* xb, R* B, R* J, R* detJac) {
    if (xb) memcpy(xb, s->xb, 3 * s->NG * sizeof(R));
    if (B) memcpy(B, s->B, 3 * s->NG * sizeof(R));
    if (J) memcpy(J, s->J, 3 * s->N * sizeof(R));
    if (detJac) memcpy(detJac, s->detJac, s->NG * sizeof(R));
}

/* k_m in the reference's kk layout: nVar values per inner point (x part, then
 * the velocity part with inertia) */
void orc_get_k(const orc_state* s, int m, R* k) {
    memcpy(k, &s->kk[(size_t)s->nVar * s->N * (size_t)m], (size_t)s->nVar * s->N * sizeof(R));
}
/* velocity at the inner points (AoS): the current one, or u_new of the last combine */
void orc_get_u(const orc_state* s, int which, R* u) { memcpy(u, which ? s->uu_new : s->uu, 3 * s->N * sizeof(R)); }
void orc_set_u(orc_state* s, const R* u) { memcpy(s->uu, u, 3 * s->N * sizeof(R)); }
void orc_get_xnew(const orc_state* s, R* xn) { memcpy(xn, s->xb_new, 3 * s->NG * sizeof(R)); }

void orc_get_scalars(const orc_state* s, double* out) {
    out[0] = s->t; out[1] = s->dt; out[2] = s->maxDelta;
    out[3] = s->timeIndex; out[4] = s->nAttempted;
}

void orc_set_time(orc_state* s, double t, double dt, int timeIndex) {
    s->t = (R)t; s->dt = (R)dt; s->timeIndex = timeIndex;
}

/* ------------------------------------------------------------------------ */
/* B = jac.B0/Delta at inner points, src/rungeKutta.cu:28-108               */
/* ------------------------------------------------------------------------ */

static void b_jac_b0(orc_state* s) {
    const P* p = &s->p;
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < p->nz; k++) {
        int i, j, l;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                R jac[3][3];
                const R* xc = s->xb;
                size_t g = GI(p, i + 1, j + 1, k + 1);
                R detJac1;
                for (l = 0; l < 3; l++) {
                    jac[l][0] = (xc[3 * GI(p, i + 2, j + 1, k + 1) + l] - xc[3 * GI(p, i, j + 1, k + 1) + l]) * p->dx1 / 2;
                    jac[l][1] = (xc[3 * GI(p, i + 1, j + 2, k + 1) + l] - xc[3 * GI(p, i + 1, j, k + 1) + l]) * p->dy1 / 2;
                    jac[l][2] = (xc[3 * GI(p, i + 1, j + 1, k + 2) + l] - xc[3 * GI(p, i + 1, j + 1, k) + l]) * p->dz1 / 2;
                }
                detJac1 = (R)(1. / (double)det3(jac));
                for (l = 0; l < 3; l++)
                    s->B[3 * g + l] = (jac[l][0] * s->B0[3 * g + 0] + jac[l][1] * s->B0[3 * g + 1] +
                                       jac[l][2] * s->B0[3 * g + 2]) * detJac1;
                s->detJac[g] = (R)(1. / (double)detJac1);
            }
    }
}

/* ------------------------------------------------------------------------ */
/* Ghost B and detJac, src/boundaries.cu:11-446                             */
/* ------------------------------------------------------------------------ */

/* addDist, src/boundaries.cu:11-35.  PI is a double constant (global.h:17),
 * so in FP32 the shear's sine argument, the sine and the product are double
 * and only the assignment to distY / distX rounds. */
static R add_dist(const P* p, int i, int j, R z, int l) {
    R x = p->dx * (R)i + p->Ox;
    R y = p->dy * (R)j + p->Oy;
    R distX = 0, distY = 0;
    if (p->initDistCode == 0) {
        distY = (R)(-p->initShearA * sin(p->initShearK * 2 * PI_D * (x + p->Ox - p->dx / 2) / (p->Lx + p->dx)) * z);
        distX = (R)(-p->initShearB * sin(p->initShearK * 2 * PI_D * (distY + y + p->Oy - p->dy / 2) / (p->Ly + p->dy)) * z);
    }
    if (p->initDistCode == 1) {
        distX = 0;
        distY = (R)(p->initShearA * REXP(-p->initShearK * x * x) * (1 - y * y) * (REXP(-1 * z + 1) - 0.15366));
    }
    return l == 0 ? distX : distY;
}

/* One ghost face pair (normal axis a: 0 = x, 1 = y, 2 = z) as updateBbound
 * does for face = a.  In-plane axes: u (block "p", 16 wide) and v ("q"). */
static void update_bbound_face(orc_state* s, int a) {
    const P* p = &s->p;
    int n3[3] = {p->nx, p->ny, p->nz};
    R d[3] = {p->dx, p->dy, p->dz};
    R d1[3] = {p->dx1, p->dy1, p->dz1};
    R L[3] = {p->Lx, p->Ly, p->Lz};
    int peri[3] = {p->xPeri, p->yPeri, p->zPeri};
    int u = (a == 0) ? 1 : 0;
    int v = (a == 2) ? 1 : 2;
    int nu_ = n3[u], nv = n3[v], na = n3[a];
    int side;
    for (side = 0; side < 2; side++) {
        int iu, iv;
        int sg = 2 * side - 1;
        for (iv = 0; iv < nv; iv++)
            for (iu = 0; iu < nu_; iu++) {
                /* ghosted coordinates of the ghost point and helpers */
                int gc[3];
                R X[3][3];        /* xbs[l][0..2] along the normal at this point */
                R Lf[3], Rt[3];   /* in-plane u neighbours */
                R Lv[3], Rv[3];   /* in-plane v neighbours */
                R B0s[3], jac[3][3], detJac1, Bv[3];
                int l;
#define PT(cu, cv, ca, out)                          \
    do {                                             \
        int c_[3];                                   \
        c_[u] = (cu); c_[v] = (cv); c_[a] = (ca);     \
        (out) = 3 * GI(p, c_[0], c_[1], c_[2]);      \
    } while (0)
                size_t q0, q1, q2, qb;
                gc[u] = iu + 1; gc[v] = iv + 1; gc[a] = side * (na + 1);
                if (!peri[a]) {
                    R zs = 0;
                    PT(iu + 1, iv + 1, side * (na + 1), q1);            /* ghost plane   */
                    PT(iu + 1, iv + 1, side == 0 ? 1 : na, q2);         /* inner plane   */
                    for (l = 0; l < 3; l++) {
                        X[l][1] = s->xb[q1 + l];
                        if (side == 0) X[l][2] = s->xb[q2 + l];
                        else X[l][0] = s->xb[q2 + l];
                    }
                    qb = q1;
                    for (l = 0; l < 3; l++) B0s[l] = s->B0[qb + l];
                    /* outer plane */
                    if (a == 2) {
                        for (l = 0; l < 2; l++)
                            X[l][2 * side] = X[l][1] - add_dist(p, iu, iv, X[2][1], l) +
                                             add_dist(p, iu, iv, 2 * p->dz * (R)sg + p->Oz + p->Lz * (R)side, l);
                        X[2][2 * side] = X[2][1] + (R)sg * p->dz;
                        zs = p->dz * (R)sg + p->Oz + p->Lz * (R)side;
                    } else {
                        for (l = 0; l < 3; l++)
                            if (l != a) X[l][2 * side] = X[l][1];
                        X[a][2 * side] = X[a][1] + (R)sg * d[a];
                    }
                    /* in-plane neighbours, extrapolated at 16-wide block edges */
                    {
                        R own[3];
                        size_t qn;
                        for (l = 0; l < 3; l++) own[l] = X[l][1];
                        /* u direction */
                        if (iu % 16 == 0) {
                            for (l = 0; l < 3; l++) Lf[l] = own[l];
                            if (a == 2) {
                                Lf[0] = own[0] - p->dx - add_dist(p, iu, iv, zs, 0) + add_dist(p, iu - 1, iv, zs, 0);
                                Lf[1] = own[1] - add_dist(p, iu, iv, zs, 1) + add_dist(p, iu - 1, iv, zs, 1);
                            } else {
                                Lf[u] = own[u] - d[u];
                            }
                        } else {
                            PT(iu, iv + 1, side * (na + 1), qn);
                            for (l = 0; l < 3; l++) Lf[l] = s->xb[qn + l];
                        }
                        if (iu % 16 == 15 || iu == nu_ - 1) {
                            for (l = 0; l < 3; l++) Rt[l] = own[l];
                            if (a == 2) {
                                Rt[0] = own[0] + p->dx - add_dist(p, iu, iv, zs, 0) + add_dist(p, iu + 1, iv, zs, 0);
                                Rt[1] = own[1] - add_dist(p, iu, iv, zs, 1) + add_dist(p, iu + 1, iv, zs, 1);
                            } else {
                                Rt[u] = own[u] + d[u];
                            }
                        } else {
                            PT(iu + 2, iv + 1, side * (na + 1), qn);
                            for (l = 0; l < 3; l++) Rt[l] = s->xb[qn + l];
                        }
                        /* v direction */
                        if (iv % 16 == 0) {
                            for (l = 0; l < 3; l++) Lv[l] = own[l];
                            if (a == 2) {
                                Lv[0] = own[0] - add_dist(p, iu, iv, zs, 0) + add_dist(p, iu, iv - 1, zs, 0);
                                Lv[1] = own[1] - p->dy - add_dist(p, iu, iv, zs, 1) + add_dist(p, iu, iv - 1, zs, 1);
                            } else {
                                Lv[v] = own[v] - d[v];
                            }
                        } else {
                            PT(iu + 1, iv, side * (na + 1), qn);
                            for (l = 0; l < 3; l++) Lv[l] = s->xb[qn + l];
                        }
                        if (iv % 16 == 15 || iv == nv - 1) {
                            for (l = 0; l < 3; l++) Rv[l] = own[l];
                            if (a == 2) {
                                Rv[0] = own[0] - add_dist(p, iu, iv, zs, 0) + add_dist(p, iu, iv + 1, zs, 0);
                                Rv[1] = own[1] + p->dy - add_dist(p, iu, iv, zs, 1) + add_dist(p, iu, iv + 1, zs, 1);
                            } else {
                                Rv[v] = own[v] + d[v];
                            }
                        } else {
                            PT(iu + 1, iv + 2, side * (na + 1), qn);
                            for (l = 0; l < 3; l++) Rv[l] = s->xb[qn + l];
                        }
                    }
                } else {
                    /* periodic: wrapped planes, shifted along the normal */
                    int pl0, pl1, pl2, pe;
                    R sh = (R)sg * (L[a] + d[a]);
                    if (side == 0) { pl0 = na - 1; pl1 = na; pl2 = 1; }
                    else { pl0 = na; pl1 = 1; pl2 = 2; }
                    PT(iu + 1, iv + 1, pl0, q0);
                    PT(iu + 1, iv + 1, pl1, q1);
                    PT(iu + 1, iv + 1, pl2, q2);
                    for (l = 0; l < 3; l++) {
                        X[l][0] = s->xb[q0 + l];
                        X[l][1] = s->xb[q1 + l];
                        X[l][2] = s->xb[q2 + l];
                    }
                    if (side == 0) {
                        X[a][0] = s->xb[q0 + a] - L[a] - d[a];
                        X[a][1] = s->xb[q1 + a] - L[a] - d[a];
                    } else {
                        X[a][1] = s->xb[q1 + a] + L[a] + d[a];
                        X[a][2] = s->xb[q2 + a] + L[a] + d[a];
                    }
                    qb = q1;
                    for (l = 0; l < 3; l++) B0s[l] = s->B0[qb + l];
                    pe = side + (1 - side) * na;
                    {
                        size_t qn;
                        /* u neighbours: block-edge threads reload from global with
                         * the shift written as x + sg*(L+d); others reuse the
                         * main load (x -/+ L -/+ d) */
                        if (iu % 16 == 0) {
                            PT(iu, iv + 1, pe, qn);
                            for (l = 0; l < 3; l++) Lf[l] = s->xb[qn + l];
                            Lf[a] = s->xb[qn + a] + sh;
                        } else {
                            PT(iu, iv + 1, pl1, qn);
                            for (l = 0; l < 3; l++) Lf[l] = s->xb[qn + l];
                            Lf[a] = side == 0 ? s->xb[qn + a] - L[a] - d[a] : s->xb[qn + a] + L[a] + d[a];
                        }
                        if (iu % 16 == 15 || iu == nu_ - 1) {
                            PT(iu + 2, iv + 1, pe, qn);
                            for (l = 0; l < 3; l++) Rt[l] = s->xb[qn + l];
                            Rt[a] = s->xb[qn + a] + sh;
                        } else {
                            PT(iu + 2, iv + 1, pl1, qn);
                            for (l = 0; l < 3; l++) Rt[l] = s->xb[qn + l];
                            Rt[a] = side == 0 ? s->xb[qn + a] - L[a] - d[a] : s->xb[qn + a] + L[a] + d[a];
                        }
                        if (iv % 16 == 0) {
                            PT(iu + 1, iv, pe, qn);
                            for (l = 0; l < 3; l++) Lv[l] = s->xb[qn + l];
                            Lv[a] = s->xb[qn + a] + sh;
                        } else {
                            PT(iu + 1, iv, pl1, qn);
                            for (l = 0; l < 3; l++) Lv[l] = s->xb[qn + l];
                            Lv[a] = side == 0 ? s->xb[qn + a] - L[a] - d[a] : s->xb[qn + a] + L[a] + d[a];
                        }
                        if (iv % 16 == 15 || iv == nv - 1) {
                            PT(iu + 1, iv + 2, pe, qn);
                            for (l = 0; l < 3; l++) Rv[l] = s->xb[qn + l];
                            Rv[a] = s->xb[qn + a] + sh;
                        } else {
                            PT(iu + 1, iv + 2, pl1, qn);
                            for (l = 0; l < 3; l++) Rv[l] = s->xb[qn + l];
                            Rv[a] = side == 0 ? s->xb[qn + a] - L[a] - d[a] : s->xb[qn + a] + L[a] + d[a];
                        }
                    }
                }
                for (l = 0; l < 3; l++) {
                    jac[l][u] = (Rt[l] - Lf[l]) * d1[u] / 2;
                    jac[l][v] = (Rv[l] - Lv[l]) * d1[v] / 2;
                    jac[l][a] = (X[l][2] - X[l][0]) * d1[a] / 2;
                }
                detJac1 = 1 / det3(jac);
                for (l = 0; l < 3; l++)
                    Bv[l] = (jac[l][0] * B0s[0] + jac[l][1] * B0s[1] + jac[l][2] * B0s[2]) * detJac1;
                if (!peri[a]) Bv[a] = B0s[a];
                {
                    size_t gq = GI(p, gc[0], gc[1], gc[2]);
                    for (l = 0; l < 3; l++) s->B[3 * gq + l] = Bv[l];
                    s->detJac[gq] = 1 / detJac1;
                }
#undef PT
            }
    }
}

/* setBbound + setPeri(B), src/main.cu:266-268, boundaries.cu:637-650 */
static void set_b_bound(orc_state* s) {
    update_bbound_face(s, 2);
    update_bbound_face(s, 1);
    update_bbound_face(s, 0);
    set_peri_field(&s->p, s->B);
}

/* setGridPeri, src/boundaries.cu:532-582 (order z, y, x) */
static void set_grid_peri(const P* p, R* xb) {
    int i, j, l;
    if (p->zPeri)
        for (i = 0; i < p->nx + 2; i++)
            for (j = 0; j < p->ny + 2; j++) {
                for (l = 0; l < 2; l++) {
                    xb[3 * GI(p, i, j, 0) + l] = xb[3 * GI(p, i, j, p->nz) + l];
                    xb[3 * GI(p, i, j, p->nz + 1) + l] = xb[3 * GI(p, i, j, 1) + l];
                }
                xb[3 * GI(p, i, j, 0) + 2] = xb[3 * GI(p, i, j, p->nz) + 2] - p->Lz - p->dz;
                xb[3 * GI(p, i, j, p->nz + 1) + 2] = xb[3 * GI(p, i, j, 1) + 2] + p->Lz + p->dz;
            }
    if (p->yPeri)
        for (i = 0; i < p->nx + 2; i++)
            for (j = 0; j < p->nz + 2; j++) {
                for (l = 0; l < 3; l += 2) {
                    xb[3 * GI(p, i, 0, j) + l] = xb[3 * GI(p, i, p->ny, j) + l];
                    xb[3 * GI(p, i, p->ny + 1, j) + l] = xb[3 * GI(p, i, 1, j) + l];
                }
                xb[3 * GI(p, i, 0, j) + 1] = xb[3 * GI(p, i, p->ny, j) + 1] - p->Ly - p->dy;
                xb[3 * GI(p, i, p->ny + 1, j) + 1] = xb[3 * GI(p, i, 1, j) + 1] + p->Ly + p->dy;
            }
    if (p->xPeri)
        for (i = 0; i < p->ny + 2; i++)
            for (j = 0; j < p->nz + 2; j++) {
                for (l = 1; l < 3; l++) {
                    xb[3 * GI(p, 0, i, j) + l] = xb[3 * GI(p, p->nx, i, j) + l];
                    xb[3 * GI(p, p->nx + 1, i, j) + l] = xb[3 * GI(p, 1, i, j) + l];
                }
                xb[3 * GI(p, 0, i, j) + 0] = xb[3 * GI(p, p->nx, i, j) + 0] - p->Lx - p->dx;
                xb[3 * GI(p, p->nx + 1, i, j) + 0] = xb[3 * GI(p, 1, i, j) + 0] + p->Lx + p->dx;
            }
}

/* ------------------------------------------------------------------------ */
/* Mimetic current, JStokes src/current.cu:222-409                          */
/* ------------------------------------------------------------------------ */

static void j_stokes(orc_state* s) {
    const P* p = &s->p;
    /* corner offsets of the three quadrilaterals (current.cu:291-382) */
    static const int Q[3][4][3] = {
        {{-1, 0, 0}, {0, -1, 0}, {1, 0, 0}, {0, 1, 0}},
        {{0, -1, 0}, {0, 0, -1}, {0, 1, 0}, {0, 0, 1}},
        {{0, 0, -1}, {-1, 0, 0}, {0, 0, 1}, {1, 0, 0}}};
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < p->nz; k++) {
        int i, j, l, m, qd, c;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                R NA[3][3], NA1[3][3], II_[3], detN, detN1;
                for (qd = 0; qd < 3; qd++) {
                    const R* xc[4];
                    const R* bc[4];
                    R dxv[4][3], cr[4][3], I = 0;
                    for (c = 0; c < 4; c++) {
                        size_t g = GI(p, i + 1 + Q[qd][c][0], j + 1 + Q[qd][c][1], k + 1 + Q[qd][c][2]);
                        xc[c] = &s->xb[3 * g];
                        bc[c] = &s->B[3 * g];
                    }
                    for (l = 0; l < 3; l++) {
                        for (c = 0; c < 4; c++) dxv[c][l] = xc[(c + 1) & 3][l] - xc[c][l];
                        I += (bc[1][l] + bc[0][l]) / 2 * dxv[0][l] + (bc[2][l] + bc[1][l]) / 2 * dxv[1][l] +
                             (bc[3][l] + bc[2][l]) / 2 * dxv[2][l] + (bc[0][l] + bc[3][l]) / 2 * dxv[3][l];
                    }
                    for (c = 0; c < 4; c++) cross3(dxv[c], dxv[(c + 1) & 3], cr[c]);
                    II_[qd] = I;
                    for (l = 0; l < 3; l++) NA[qd][l] = (cr[0][l] + cr[1][l] + cr[2][l] + cr[3][l]) / 4;
                }
                detN = det3(NA);
                detN1 = 1 / detN;
                NA1[0][0] = (NA[1][1] * NA[2][2] - NA[1][2] * NA[2][1]) * detN1;
                NA1[0][1] = (NA[0][2] * NA[2][1] - NA[0][1] * NA[2][2]) * detN1;
                NA1[0][2] = (NA[0][1] * NA[1][2] - NA[0][2] * NA[1][1]) * detN1;
                NA1[1][0] = (NA[1][2] * NA[2][0] - NA[1][0] * NA[2][2]) * detN1;
                NA1[1][1] = (NA[0][0] * NA[2][2] - NA[0][2] * NA[2][0]) * detN1;
                NA1[1][2] = (NA[0][2] * NA[1][0] - NA[0][0] * NA[1][2]) * detN1;
                NA1[2][0] = (NA[1][0] * NA[2][1] - NA[1][1] * NA[2][0]) * detN1;
                NA1[2][1] = (NA[0][1] * NA[2][0] - NA[0][0] * NA[2][1]) * detN1;
                NA1[2][2] = (NA[0][0] * NA[1][1] - NA[0][1] * NA[1][0]) * detN1;
                for (l = 0; l < 3; l++) {
                    R Jl = 0;
                    for (m = 0; m < 3; m++) Jl += NA1[l][m] * II_[m];
                    s->J[3 * II(p, i, j, k) + l] = Jl;
                }
            }
    }
}

/* ------------------------------------------------------------------------ */
/* Octilateral Stokes current, JStokes4th src/current.cu:413-736            */
/* ------------------------------------------------------------------------ */

/* For each of the three planes through the point (axes (u, v) = (x, y),
 * (y, z), (z, x)), the contour through the eight neighbours P(a, b),
 * a, b in {-1, 0, 1} along u and v, in the order (-1,-1) (0,-1) (1,-1) (1,0)
 * (1,1) (0,1) (-1,1) (-1,0): the circulation sum (B_end + B_start)/2 . dx over
 * its eight edges, and the area vector (1/2) sum of the corner cross products
 * dx2 x dx3 + dx4 x dx5 + dx6 x dx7 + dx8 x dx1 plus (1/4) that of the inner
 * diamond through the face neighbours (current.cu:513-736); J solves the 3x3
 * system as JStokes does, dividing by the determinant. */
static void j_stokes4th(orc_state* s) {
    const P* p = &s->p;
    static const int ax[3][2] = {{0, 1}, {1, 2}, {2, 0}};
    static const int ring[9][2] = {{0, 0}, {1, 0}, {2, 0}, {2, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}, {0, 0}};
    static const int dia[5][2] = {{0, 1}, {1, 0}, {2, 1}, {1, 2}, {0, 1}};   /* dxA..dxD */
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < p->nz; k++) {
        int i, j, l, m, pl, e;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                R NA[3][3], NA1[3][3], II_[3], detNA;
                for (pl = 0; pl < 3; pl++) {
                    const R* X[9];
                    const R* Bp[9];
                    R dx[8][3], dd[4][3], I = 0, c[4][3];
                    for (e = 0; e < 8; e++) {
                        int o[3] = {0, 0, 0};
                        o[ax[pl][0]] = ring[e][0] - 1;
                        o[ax[pl][1]] = ring[e][1] - 1;
                        {
                            const size_t g = GI(p, i + 1 + o[0], j + 1 + o[1], k + 1 + o[2]);
                            X[e] = &s->xb[3 * g];
                            Bp[e] = &s->B[3 * g];
                        }
                    }
                    X[8] = X[0]; Bp[8] = Bp[0];
                    for (l = 0; l < 3; l++) {
                        for (e = 0; e < 8; e++) dx[e][l] = X[e + 1][l] - X[e][l];
                        I += (Bp[1][l] + Bp[0][l]) / 2 * dx[0][l] + (Bp[2][l] + Bp[1][l]) / 2 * dx[1][l] +
                             (Bp[3][l] + Bp[2][l]) / 2 * dx[2][l] + (Bp[4][l] + Bp[3][l]) / 2 * dx[3][l] +
                             (Bp[5][l] + Bp[4][l]) / 2 * dx[4][l] + (Bp[6][l] + Bp[5][l]) / 2 * dx[5][l] +
                             (Bp[7][l] + Bp[6][l]) / 2 * dx[6][l] + (Bp[8][l] + Bp[7][l]) / 2 * dx[7][l];
                    }
                    /* the inner diamond: dxA..dxD between the face neighbours */
                    for (e = 0; e < 4; e++) {
                        int o0[3] = {0, 0, 0}, o1[3] = {0, 0, 0};
                        o0[ax[pl][0]] = dia[e][0] - 1; o0[ax[pl][1]] = dia[e][1] - 1;
                        o1[ax[pl][0]] = dia[e + 1][0] - 1; o1[ax[pl][1]] = dia[e + 1][1] - 1;
                        {
                            const R* a = &s->xb[3 * GI(p, i + 1 + o0[0], j + 1 + o0[1], k + 1 + o0[2])];
                            const R* b = &s->xb[3 * GI(p, i + 1 + o1[0], j + 1 + o1[1], k + 1 + o1[2])];
                            for (l = 0; l < 3; l++) dd[e][l] = b[l] - a[l];
                        }
                    }
                    II_[pl] = I;
                    cross3(dx[1], dx[2], c[0]);
                    cross3(dx[3], dx[4], c[1]);
                    cross3(dx[5], dx[6], c[2]);
                    cross3(dx[7], dx[0], c[3]);
                    for (l = 0; l < 3; l++) NA[pl][l] = (c[0][l] + c[1][l] + c[2][l] + c[3][l]) / 2;
                    cross3(dd[0], dd[1], c[0]);
                    cross3(dd[1], dd[2], c[1]);
                    cross3(dd[2], dd[3], c[2]);
                    cross3(dd[3], dd[0], c[3]);
                    for (l = 0; l < 3; l++) NA[pl][l] += (c[0][l] + c[1][l] + c[2][l] + c[3][l]) / 4;
                }
                detNA = NA[0][0] * NA[1][1] * NA[2][2] + NA[0][1] * NA[1][2] * NA[2][0] + NA[0][2] * NA[1][0] * NA[2][1] -
                        NA[0][0] * NA[1][2] * NA[2][1] - NA[0][1] * NA[1][0] * NA[2][2] - NA[0][2] * NA[1][1] * NA[2][0];
                NA1[0][0] = (NA[1][1] * NA[2][2] - NA[1][2] * NA[2][1]) / detNA;
                NA1[0][1] = (NA[0][2] * NA[2][1] - NA[0][1] * NA[2][2]) / detNA;
                NA1[0][2] = (NA[0][1] * NA[1][2] - NA[0][2] * NA[1][1]) / detNA;
                NA1[1][0] = (NA[1][2] * NA[2][0] - NA[1][0] * NA[2][2]) / detNA;
                NA1[1][1] = (NA[0][0] * NA[2][2] - NA[0][2] * NA[2][0]) / detNA;
                NA1[1][2] = (NA[0][2] * NA[1][0] - NA[0][0] * NA[1][2]) / detNA;
                NA1[2][0] = (NA[1][0] * NA[2][1] - NA[1][1] * NA[2][0]) / detNA;
                NA1[2][1] = (NA[0][1] * NA[2][0] - NA[0][0] * NA[2][1]) / detNA;
                NA1[2][2] = (NA[0][0] * NA[1][1] - NA[0][1] * NA[1][0]) / detNA;
                for (l = 0; l < 3; l++) {
                    R Jl = 0;
                    for (m = 0; m < 3; m++) Jl += NA1[l][m] * II_[m];
                    s->J[3 * II(p, i, j, k) + l] = Jl;
                }
            }
    }
}

/* ------------------------------------------------------------------------ */
/* Quintilateral Stokes current, JStokesQuint src/current.cu:737-1199       */
/* ------------------------------------------------------------------------ */

/* For each plane through the point, axes (u, v, w) = (x, y, z), (y, z, x),
 * (z, x, y), with P(a, b) the in-plane neighbour at offsets (a - 1, b - 1):
 * the diamond through the face neighbours P(0,1) P(1,0) P(2,1) P(1,2), and,
 * when the orientation tests of current.cu:863-896 pick a corner triangle,
 * that triangle's two outer edges in place of one diamond edge.  The tests
 * are restated as written: each later test looks at the edge vectors the
 * previous one stored, the third compares with 4 instead of 0, the first
 * triangle's edges take the B averages of the other edge (current.cu:919-
 * 922), and in the second and third planes the fourth triangle's second edge
 * runs from P(1, 2), not P(0, 2), to P(0, 1) (current.cu:995-996,
 * 1104-1105).  Area vector: (1/4) of the diamond's consecutive cross
 * products plus (1/2) of the triangle's; the solve multiplies by 1/det.
 *
 * With tri_only set, the triangular Stokes current (JStokesTri,
 * current.cu:1202-1681): the same tests, but a plane where they pick a
 * triangle takes that triangle alone, its two outer edges and the reversed
 * diamond edge (with that edge's B average) as the contour and (1/2) of the
 * outer edges' cross product as the area vector.  The reference adds that
 * half cross product to an area vector that nothing set before
 * (current.cu:1420-1424); its compiled kernel returns NaN in all three
 * components of J at every point where a plane takes a triangle (measured on
 * a grid with 618 such points out of 3468), so that unset start is NaN here. */
static void j_stokes_quint(orc_state* s, int tri_only) {
    const P* p = &s->p;
    static const int ax[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < p->nz; k++) {
        int i, j, l, m, pl;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                R NA[3][3], NA1[3][3], II_[3], detN, detN1;
                for (pl = 0; pl < 3; pl++) {
#define PO(a_, b_, w_, out)                                                   \
    do {                                                                      \
        int o_[3] = {0, 0, 0};                                                \
        o_[ax[pl][0]] = (a_) - 1; o_[ax[pl][1]] = (b_) - 1; o_[ax[pl][2]] = (w_); \
        (out) = GI(p, i + 1 + o_[0], j + 1 + o_[1], k + 1 + o_[2]);          \
    } while (0)
                    size_t g;
                    const R *xc, *x[3][3], *xw_p, *xw_m, *b[3][3];
                    R dx1[3], dx2[3], dx3[3], dx4[3], dx5[3], dx6[3], c[3], I = 0;
                    int a, bb, tri = 0;
                    for (a = 0; a < 3; a++)
                        for (bb = 0; bb < 3; bb++) {
                            PO(a, bb, 0, g);
                            x[a][bb] = &s->xb[3 * g];
                            b[a][bb] = &s->B[3 * g];
                        }
                    xc = x[1][1];
                    PO(1, 1, 1, g); xw_p = &s->xb[3 * g];
                    PO(1, 1, -1, g); xw_m = &s->xb[3 * g];
#undef PO
                    for (l = 0; l < 3; l++) {
                        dx1[l] = x[1][0][l] - xc[l];
                        dx2[l] = x[2][1][l] - xc[l];
                        dx3[l] = x[1][2][l] - xc[l];
                        dx4[l] = x[0][1][l] - xc[l];
                        dx5[l] = xw_p[l] - xc[l];
                        dx6[l] = xw_m[l] - xc[l];
                    }
                    cross3(dx1, dx2, c);
                    if (dot3(c, dx5) < 0 || dot3(c, dx6) > 0) {
                        for (l = 0; l < 3; l++) {
                            dx5[l] = x[2][0][l] - x[1][0][l];
                            dx6[l] = x[2][1][l] - x[2][0][l];
                        }
                        tri = 2;
                    }
                    if (tri != 0) {
                        cross3(dx2, dx3, c);
                        if (dot3(c, dx5) < 0 || dot3(c, dx6) > 0) {
                            for (l = 0; l < 3; l++) {
                                dx5[l] = x[2][2][l] - x[2][1][l];
                                dx6[l] = x[1][2][l] - x[2][2][l];
                            }
                            tri = 3;
                        }
                    }
                    if (tri != 0) {
                        cross3(dx3, dx4, c);
                        if (dot3(c, dx5) < 0 || dot3(c, dx6) > 4) {
                            for (l = 0; l < 3; l++) {
                                dx5[l] = x[0][2][l] - x[1][2][l];
                                dx6[l] = x[0][1][l] - (pl == 0 ? x[0][2][l] : x[1][2][l]);
                            }
                            tri = 4;
                        }
                    }
                    cross3(dx4, dx1, c);
                    if (tri != 0) {
                        if (dot3(c, dx5) < 0 || dot3(c, dx6) > 0) {
                            for (l = 0; l < 3; l++) {
                                dx5[l] = x[1][0][l] - x[0][0][l];
                                dx6[l] = x[0][0][l] - x[0][1][l];
                            }
                            tri = 1;
                        }
                    }
                    for (l = 0; l < 3; l++) {
                        dx1[l] = x[1][0][l] - x[0][1][l];
                        dx2[l] = x[2][1][l] - x[1][0][l];
                        dx3[l] = x[1][2][l] - x[2][1][l];
                        dx4[l] = x[0][1][l] - x[1][2][l];
                        if (tri_only && tri != 0) {
                            /* the triangle's closing edge: the diamond edge reversed */
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
                        if (tri == 1)
                            I += (b[0][1][l] + b[0][0][l]) / 2 * dx5[l] + (b[1][0][l] + b[0][0][l]) / 2 * dx6[l];
                        if (tri == 2)
                            I += (b[1][0][l] + b[2][0][l]) / 2 * dx5[l] + (b[2][1][l] + b[2][0][l]) / 2 * dx6[l];
                        if (tri == 3)
                            I += (b[2][1][l] + b[2][2][l]) / 2 * dx5[l] + (b[1][2][l] + b[2][2][l]) / 2 * dx6[l];
                        if (tri == 4)
                            I += (b[1][2][l] + b[0][2][l]) / 2 * dx5[l] + (b[0][1][l] + b[0][2][l]) / 2 * dx6[l];
                    }
                    {
                        R c12[3], c23[3], c34[3], c41[3], c56[3];
                        cross3(dx1, dx2, c12);
                        cross3(dx2, dx3, c23);
                        cross3(dx3, dx4, c34);
                        cross3(dx4, dx1, c41);
                        if (tri > 0) cross3(dx5, dx6, c56);
                        II_[pl] = I;
                        for (l = 0; l < 3; l++) {
                            if (tri_only && tri > 0) {
                                NA[pl][l] = (R)NAN + c56[l] / 2;
                            } else {
                                NA[pl][l] = (c12[l] + c23[l] + c34[l] + c41[l]) / 4;
                                if (tri > 0) NA[pl][l] += c56[l] / 2;
                            }
                        }
                    }
                }
                detN = NA[0][0] * NA[1][1] * NA[2][2] + NA[0][1] * NA[1][2] * NA[2][0] + NA[0][2] * NA[1][0] * NA[2][1] -
                       NA[0][0] * NA[1][2] * NA[2][1] - NA[0][1] * NA[1][0] * NA[2][2] - NA[0][2] * NA[1][1] * NA[2][0];
                detN1 = 1 / detN;
                NA1[0][0] = (NA[1][1] * NA[2][2] - NA[1][2] * NA[2][1]) * detN1;
                NA1[0][1] = (NA[0][2] * NA[2][1] - NA[0][1] * NA[2][2]) * detN1;
                NA1[0][2] = (NA[0][1] * NA[1][2] - NA[0][2] * NA[1][1]) * detN1;
                NA1[1][0] = (NA[1][2] * NA[2][0] - NA[1][0] * NA[2][2]) * detN1;
                NA1[1][1] = (NA[0][0] * NA[2][2] - NA[0][2] * NA[2][0]) * detN1;
                NA1[1][2] = (NA[0][2] * NA[1][0] - NA[0][0] * NA[1][2]) * detN1;
                NA1[2][0] = (NA[1][0] * NA[2][1] - NA[1][1] * NA[2][0]) * detN1;
                NA1[2][1] = (NA[0][1] * NA[2][0] - NA[0][0] * NA[2][1]) * detN1;
                NA1[2][2] = (NA[0][0] * NA[1][1] - NA[0][1] * NA[1][0]) * detN1;
                for (l = 0; l < 3; l++) {
                    R Jl = 0;
                    for (m = 0; m < 3; m++) Jl += NA1[l][m] * II_[m];
                    s->J[3 * II(p, i, j, k) + l] = Jl;
                }
            }
    }
}

/* ------------------------------------------------------------------------ */
/* Finite-difference current, JClassic src/current.cu:10-218                */
/* ------------------------------------------------------------------------ */

/* J = curl B with B = jac.B0 / Delta, differentiated by the chain rule on the
 * initial grid: d B_k / d X_a = sum_b (d2x[k][a][b] B0_b det1
 * + jac[k][b] dB0[b][a] det1 + jac[k][b] B0_b d det1 / d X_a) and
 * d / d x_c = sum_a jac1[a][c] d / d X_a (current.cu:142-216).  B itself is
 * not read: the inputs are x (with its edge neighbours), B0 and detJac at
 * the point and its six face neighbours (ghost values included). */
static void j_classic(orc_state* s) {
    const P* p = &s->p;
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < p->nz; k++) {
        int i, j, l, a, b;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                R jac[3][3], jac1[3][3], d2[3][3][3], dB0[3][3], dDet1[3], det1, B0l[3], Jv[3];
                const R* x = s->xb;
#define XV(di, dj, dk, l_) x[3 * GI(p, i + 1 + (di), j + 1 + (dj), k + 1 + (dk)) + (l_)]
#define B0V(di, dj, dk, l_) s->B0[3 * GI(p, i + 1 + (di), j + 1 + (dj), k + 1 + (dk)) + (l_)]
#define DV(di, dj, dk) s->detJac[GI(p, i + 1 + (di), j + 1 + (dj), k + 1 + (dk))]
                for (l = 0; l < 3; l++) {
                    jac[l][0] = (XV(1, 0, 0, l) - XV(-1, 0, 0, l)) * p->dx1 / 2;
                    jac[l][1] = (XV(0, 1, 0, l) - XV(0, -1, 0, l)) * p->dy1 / 2;
                    jac[l][2] = (XV(0, 0, 1, l) - XV(0, 0, -1, l)) * p->dz1 / 2;
                    B0l[l] = B0V(0, 0, 0, l);
                }
                det1 = 1 / DV(0, 0, 0);
                jac1[0][0] = (jac[1][1] * jac[2][2] - jac[1][2] * jac[2][1]) * det1;
                jac1[0][1] = (jac[0][2] * jac[2][1] - jac[0][1] * jac[2][2]) * det1;
                jac1[0][2] = (jac[0][1] * jac[1][2] - jac[0][2] * jac[1][1]) * det1;
                jac1[1][0] = (jac[1][2] * jac[2][0] - jac[1][0] * jac[2][2]) * det1;
                jac1[1][1] = (jac[0][0] * jac[2][2] - jac[0][2] * jac[2][0]) * det1;
                jac1[1][2] = (jac[0][2] * jac[1][0] - jac[0][0] * jac[1][2]) * det1;
                jac1[2][0] = (jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0]) * det1;
                jac1[2][1] = (jac[0][1] * jac[2][0] - jac[0][0] * jac[2][1]) * det1;
                jac1[2][2] = (jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0]) * det1;
                for (l = 0; l < 3; l++) {
                    d2[l][0][0] = (XV(1, 0, 0, l) - 2 * XV(0, 0, 0, l) + XV(-1, 0, 0, l)) * p->dx1 * p->dx1;
                    d2[l][1][1] = (XV(0, 1, 0, l) - 2 * XV(0, 0, 0, l) + XV(0, -1, 0, l)) * p->dy1 * p->dy1;
                    d2[l][2][2] = (XV(0, 0, 1, l) - 2 * XV(0, 0, 0, l) + XV(0, 0, -1, l)) * p->dz1 * p->dz1;
                    d2[l][0][1] = (XV(1, 1, 0, l) - XV(1, -1, 0, l) - XV(-1, 1, 0, l) + XV(-1, -1, 0, l)) * p->dx1 * p->dy1 / 4;
                    d2[l][0][2] = (XV(1, 0, 1, l) - XV(1, 0, -1, l) - XV(-1, 0, 1, l) + XV(-1, 0, -1, l)) * p->dx1 * p->dz1 / 4;
                    d2[l][1][2] = (XV(0, 1, 1, l) - XV(0, -1, 1, l) - XV(0, 1, -1, l) + XV(0, -1, -1, l)) * p->dy1 * p->dz1 / 4;
                    d2[l][1][0] = d2[l][0][1];
                    d2[l][2][0] = d2[l][0][2];
                    d2[l][2][1] = d2[l][1][2];
                    dB0[l][0] = (B0V(1, 0, 0, l) - B0V(-1, 0, 0, l)) * p->dx1 / 2;
                    dB0[l][1] = (B0V(0, 1, 0, l) - B0V(0, -1, 0, l)) * p->dy1 / 2;
                    dB0[l][2] = (B0V(0, 0, 1, l) - B0V(0, 0, -1, l)) * p->dz1 / 2;
                }
                dDet1[0] = (1 / DV(1, 0, 0) - 1 / DV(-1, 0, 0)) * p->dx1 / 2;
                dDet1[1] = (1 / DV(0, 1, 0) - 1 / DV(0, -1, 0)) * p->dy1 / 2;
                dDet1[2] = (1 / DV(0, 0, 1) - 1 / DV(0, 0, -1)) * p->dz1 / 2;
#undef XV
#undef B0V
#undef DV
                Jv[0] = 0; Jv[1] = 0; Jv[2] = 0;
                for (a = 0; a < 3; a++)
                    for (b = 0; b < 3; b++) {
                        /* d B_m / d X_a, term b, for m = 0, 1, 2 */
                        R dB[3];
                        for (l = 0; l < 3; l++)
                            dB[l] = d2[l][a][b] * B0l[b] * det1 + jac[l][b] * dB0[b][a] * det1 + jac[l][b] * B0l[b] * dDet1[a];
                        Jv[0] += jac1[a][1] * dB[2] - jac1[a][2] * dB[1];
                        Jv[1] += jac1[a][2] * dB[0] - jac1[a][0] * dB[2];
                        Jv[2] += jac1[a][0] * dB[1] - jac1[a][1] * dB[0];
                    }
                for (l = 0; l < 3; l++) s->J[3 * II(p, i, j, k) + l] = Jv[l];
            }
    }
}

/* ------------------------------------------------------------------------ */
/* Pressure gradient, gradPClassic src/gradP.cu:10-156                      */
/* ------------------------------------------------------------------------ */

static void grad_p(orc_state* s) {
    const P* p = &s->p;
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < p->nz; k++) {
        int i, j, l, a, b;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                R jac[3][3], jac1[3][3], d2[3][3][3], det1, g[3];
                const R* x = s->xb;
#define XV(di, dj, dk, l_) x[3 * GI(p, i + 1 + (di), j + 1 + (dj), k + 1 + (dk)) + (l_)]
                det1 = 1 / s->detJac[GI(p, i + 1, j + 1, k + 1)];
                for (l = 0; l < 3; l++) {
                    jac[l][0] = (XV(1, 0, 0, l) - XV(-1, 0, 0, l)) * p->dx1 / 2;
                    jac[l][1] = (XV(0, 1, 0, l) - XV(0, -1, 0, l)) * p->dy1 / 2;
                    jac[l][2] = (XV(0, 0, 1, l) - XV(0, 0, -1, l)) * p->dz1 / 2;
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
                for (l = 0; l < 3; l++) {
                    d2[l][0][0] = (XV(1, 0, 0, l) - 2 * XV(0, 0, 0, l) + XV(-1, 0, 0, l)) * p->dx1 * p->dx1;
                    d2[l][1][1] = (XV(0, 1, 0, l) - 2 * XV(0, 0, 0, l) + XV(0, -1, 0, l)) * p->dy1 * p->dy1;
                    d2[l][2][2] = (XV(0, 0, 1, l) - 2 * XV(0, 0, 0, l) + XV(0, 0, -1, l)) * p->dz1 * p->dz1;
                    d2[l][0][1] = (XV(1, 1, 0, l) - XV(1, -1, 0, l) - XV(-1, 1, 0, l) + XV(-1, -1, 0, l)) * p->dx1 * p->dy1 / 4;
                    d2[l][0][2] = (XV(1, 0, 1, l) - XV(1, 0, -1, l) - XV(-1, 0, 1, l) + XV(-1, 0, -1, l)) * p->dx1 * p->dz1 / 4;
                    d2[l][1][2] = (XV(0, 1, 1, l) - XV(0, -1, 1, l) - XV(0, 1, -1, l) + XV(0, -1, -1, l)) * p->dy1 * p->dz1 / 4;
                    d2[l][1][0] = d2[l][0][1];
                    d2[l][2][0] = d2[l][0][2];
                    d2[l][2][1] = d2[l][1][2];
                }
#undef XV
                g[0] = 0; g[1] = 0; g[2] = 0;
                for (a = 0; a < 3; a++)
                    for (b = 0; b < 3; b++)
                        for (l = 0; l < 3; l++) {
                            g[0] -= d2[a][b][l] * jac1[b][a] * jac1[l][0];
                            g[1] -= d2[a][b][l] * jac1[b][a] * jac1[l][1];
                            g[2] -= d2[a][b][l] * jac1[b][a] * jac1[l][2];
                        }
                if (p->p0Amp != 0) {
                    /* This library's extension (no reference counterpart):
                     * p = p0(X) / Delta with p0(X) = beta (1 + p0Amp exp(-(X^2 + Y^2) / p0Width^2))
                     * on the initial grid, so grad_x p = p0 grad_x(1/Delta) + (1/Delta) grad_x p0,
                     * where grad_x(1/Delta) = det1 * g (the sum above) and
                     * d p0 / d x_c = sum_a d p0 / d X_a  d X_a / d x_c = sum_a dp0_a jac1[a][c]. */
                    const R X = p->dx * (R)i + p->Ox, Y = p->dy * (R)j + p->Oy;
                    const R w2 = (R)((double)p->p0Width * (double)p->p0Width);
                    const R e = p->p0Amp * (R)exp((double)(-(X * X + Y * Y) / w2));
                    const R p0 = p->beta * (1 + e);
                    const R dp0x = p->beta * e * (-2 * X / w2), dp0y = p->beta * e * (-2 * Y / w2);
                    for (l = 0; l < 3; l++) {
                        g[l] = (p0 * g[l] + dp0x * jac1[0][l] + dp0y * jac1[1][l]) * det1;
                        s->gradP[3 * II(p, i, j, k) + l] = g[l];
                    }
                } else {
                    for (l = 0; l < 3; l++) {
                        g[l] *= p->beta * det1;
                        s->gradP[3 * II(p, i, j, k) + l] = g[l];
                    }
                }
            }
    }
}

/* jxbAver, src/rungeKutta.cu:357-443: J x B at the six face neighbours
 * (zero beyond the inner range), each scaled by jxbAverWeight / 6.  J is the
 * current stage's inner J, B the ghosted B of the stage; the +z neighbour's B
 * is read with the reference's plane stride (nx+1)(ny+1) (rungeKutta.cu:428),
 * which lands on another point of the array. */
static void jxb_aver(const orc_state* s, int i, int j, int k, R jxb[6][3]) {
    const P* p = &s->p;
    const size_t nx = (size_t)p->nx, ny = (size_t)p->ny;
    const R w6 = p->jxbAverWeight / 6;
    int m, l;
    for (m = 0; m < 6; m++) {
        const R* J = NULL;
        const R* B = NULL;
        switch (m) {
            case 0: if (i > 0) { J = &s->J[3 * II(p, i - 1, j, k)]; B = &s->B[3 * GI(p, i, j + 1, k + 1)]; } break;
            case 1: if (i < p->nx - 1) { J = &s->J[3 * II(p, i + 1, j, k)]; B = &s->B[3 * GI(p, i + 2, j + 1, k + 1)]; } break;
            case 2: if (j > 0) { J = &s->J[3 * II(p, i, j - 1, k)]; B = &s->B[3 * GI(p, i + 1, j, k + 1)]; } break;
            case 3: if (j < p->ny - 1) { J = &s->J[3 * II(p, i, j + 1, k)]; B = &s->B[3 * GI(p, i + 1, j + 2, k + 1)]; } break;
            case 4: if (k > 0) { J = &s->J[3 * II(p, i, j, k - 1)]; B = &s->B[3 * GI(p, i + 1, j + 1, k)]; } break;
            default:
                if (k < p->nz - 1) {
                    J = &s->J[3 * II(p, i, j, k + 1)];
                    B = &s->B[3 * ((size_t)(i + 1) + (nx + 2) * (size_t)(j + 1) + (size_t)(k + 2) * (nx + 1) * (ny + 1))];
                }
        }
        if (J) cross3(J, B, jxb[m]);
        else jxb[m][0] = jxb[m][1] = jxb[m][2] = 0;
        for (l = 0; l < 3; l++) jxb[m][l] *= w6;
    }
}

/* epsilon profile, src/rungeKutta.cu:180-185 (evaluated in double) */
static R eps_profile(const P* p, int i, int j, int k) {
    if (!p->epsilonProf) return 1;
    return (R)((-(i - (p->nx) / 2.) / (p->nx) * (i + 1 - (p->nx) / 2.) / (p->nx) * 4 + 1) *
               (-(j - (p->ny) / 2.) / (p->ny) * (j + 1 - (p->ny) / 2.) / (p->ny) * 4 + 1) *
               (-(k - (p->nz) / 2.) / (p->nz) * (k + 1 - (p->nz) / 2.) / (p->nz) * 4 + 1));
}

/* ------------------------------------------------------------------------ */
/* Stage increment and incremental stage position, kk src/rungeKutta.cu:112-247 */
/* ------------------------------------------------------------------------ */

static void kk_stage(orc_state* s, int n, R dt) {
    const P* p = &s->p;
    int k;
    size_t N = s->N;
#pragma omp parallel for schedule(static)
    for (k = 0; k < p->nz; k++) {
        int i, j, l, m;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                size_t g = GI(p, i + 1, j + 1, k + 1), q = II(p, i, j, k);
                const int nV = s->nVar;
                R kn[6], xs[3], epsilon;
                if (!p->inertia) {
                    cross3(&s->J[3 * q], &s->B[3 * g], kn);
                    if (p->jxbAver) {
                        /* rungeKutta.cu:172-178 */
                        R jxb[6][3];
                        jxb_aver(s, i, j, k, jxb);
                        for (l = 0; l < 3; l++) {
                            kn[l] *= (1 - p->jxbAverWeight);
                            for (m = 0; m < 6; m++) kn[l] += jxb[m][l];
                        }
                    }
                    epsilon = eps_profile(p, i, j, k);
                    for (l = 0; l < 3; l++) {
                        kn[l] *= dt * epsilon;
                        if (p->pressure) kn[l] += -dt * s->gradP[3 * q + l];
                    }
                } else {
                    /* rungeKutta.cu:195-212: k_x = dt u, k_u = dt Delta (J x B)
                     * - dt nu u Delta - dt grad p (no epsilon profile) */
                    const R D = s->detJac[g];
                    cross3(&s->J[3 * q], &s->B[3 * g], &kn[3]);
                    for (l = 0; l < 3; l++) {
                        const R u = s->uu[3 * q + l];
                        kn[l] = dt * u;
                        kn[3 + l] *= dt * D;
                        kn[3 + l] -= dt * p->nu * u * D;
                        if (p->pressure) kn[3 + l] += -dt * s->gradP[3 * q + l];
                    }
                }
                for (l = 0; l < nV; l++) s->kk[(size_t)nV * (N * (size_t)n + q) + l] = kn[l];
                for (l = 0; l < 3; l++) {
                    xs[l] = s->xb[3 * g + l];
                    for (m = 0; m < n + 1; m++)
                        xs[l] += (s->b[n + 1][m] - s->b[n][m]) * s->kk[(size_t)nV * (N * (size_t)m + q) + l];
                    s->xb_tmp[3 * g + l] = xs[l];
                }
                if (p->inertia)
                    for (l = 0; l < 3; l++) {
                        R us = s->uu[3 * q + l];
                        for (m = 0; m < n + 1; m++)
                            us += (s->b[n + 1][m] - s->b[n][m]) * s->kk[(size_t)nV * (N * (size_t)m + q) + 3 + l];
                        s->uu_tmp[3 * q + l] = us;
                    }
            }
    }
}

/* x_new, x* and the error norm, xNewStar src/rungeKutta.cu:251-353 */
static void x_new_star(orc_state* s) {
    const P* p = &s->p;
    size_t N = s->N;
    int k;
    R gmax = 0;
#pragma omp parallel for schedule(static) reduction(max : gmax)
    for (k = 0; k < p->nz; k++) {
        int i, j, l, n;
        R lmax = 0;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                size_t g = GI(p, i + 1, j + 1, k + 1), q = II(p, i, j, k);
                const size_t nV = (size_t)s->nVar;
                for (l = 0; l < 3; l++) {
                    R xn = s->xb[3 * g + l], xs = s->xb[3 * g + l], dl;
                    if (l < 2 || p->zUpdate) {
                        if (p->errMode == 0) {
                            for (n = 0; n < 6; n++) {
                                xn += s->c[n] * s->kk[nV * (N * (size_t)n + q) + l];
                                xs += s->cs[n] * s->kk[nV * (N * (size_t)n + q) + l];
                            }
                            dl = (R)fabs((double)(xn - xs));
                        } else {
                            double e = 0;
                            for (n = 0; n < 6; n++) {
                                xn += s->c[n] * s->kk[nV * (N * (size_t)n + q) + l];
                                e += ((double)s->c[n] - (double)s->cs[n]) * (double)s->kk[nV * (N * (size_t)n + q) + l];
                            }
                            dl = (R)fabs(e);
                        }
                    } else {
                        dl = 0;
                    }
                    s->xb_new[3 * g + l] = xn;
                    if (dl > lmax) lmax = dl;   /* maxValue semantics: NaN never wins */
                }
                /* u_new = u + sum c k_u (rungeKutta.cu:311-322); the error is x's only */
                if (p->inertia)
                    for (l = 0; l < 3; l++) {
                        R un = s->uu[3 * q + l];
                        for (n = 0; n < 6; n++) un += s->c[n] * s->kk[nV * (N * (size_t)n + q) + 3 + l];
                        s->uu_new[3 * q + l] = un;
                    }
            }
        if (lmax > gmax) gmax = lmax;
    }
    s->maxDelta = gmax;
}

/* ------------------------------------------------------------------------ */
/* Public stage / step API                                                   */
/* ------------------------------------------------------------------------ */

/* B, ghosts and J at the current grid (main.cu:262-272 and 343-353). */
void orc_refresh_fields(orc_state* s) {
    b_jac_b0(s);
    set_b_bound(s);
    if (s->p.jClassic) j_classic(s);
    else if (s->p.jOct) j_stokes4th(s);
    else if (s->p.jQuint) j_stokes_quint(s, 0);
    else if (s->p.jTri) j_stokes_quint(s, 1);
    else j_stokes(s);
}

/* One RK stage n, src/main.cu:260-307. */
void orc_stage(orc_state* s, int n) {
    orc_refresh_fields(s);
    if (s->p.pressure) grad_p(s);
    kk_stage(s, n, s->dt);
    set_grid_peri(&s->p, s->xb_tmp);
    memcpy(s->xb, s->xb_tmp, 3 * s->NG * sizeof(R));
    if (s->p.inertia) memcpy(s->uu, s->uu_tmp, 3 * s->N * sizeof(R));   /* main.cu:296-305 */
}

/* xNewStar + setGridPeri(xb_new), src/main.cu:309-315. */
void orc_combine(orc_state* s) {
    x_new_star(s);
    set_grid_peri(&s->p, s->xb_new);
}

/* One attempted step, src/main.cu:259-384 without diagnostics or dumps.
 * Returns 1 if accepted, 0 if rejected, -1 if the loop condition already
 * fails (timeIndex >= nCycle or dt <= dtMin). */
int orc_step(orc_state* s, int nCycle) {
    int n;
    const P* p = &s->p;
    if (!(s->timeIndex < nCycle && s->dt > p->dtMin)) return -1;
    for (n = 0; n < 6; n++) orc_stage(s, n);
    orc_combine(s);
    s->nAttempted++;
    if (s->maxDelta < p->maxError) {
        s->t += s->dt;
        memcpy(s->xb, s->xb_new, 3 * s->NG * sizeof(R));
        if (p->inertia) memcpy(s->uu, s->uu_new, 3 * s->N * sizeof(R));   /* main.cu:331-339 */
        orc_refresh_fields(s);
        if (s->maxDelta > 0) s->dt = (R)((double)s->dt * pow(0.9 * (double)p->maxError / (double)s->maxDelta, (double)(R)0.2));
        s->timeIndex++;
        return 1;
    }
    if (s->maxDelta > 0) s->dt = (R)((double)s->dt * pow(0.9 * (double)p->maxError / (double)s->maxDelta, (double)(R)0.2));
    return 0;
}

/* Run steps until nCycle accepted steps or dt <= dtMin or maxAttempts.
 * Logs (maxDelta, dt after update, accepted) per attempt into log[3*a]. */
int orc_run(orc_state* s, int nCycle, int maxAttempts, double* log) {
    int a = 0;
    while (a < maxAttempts) {
        R dtBefore = s->dt;
        int r = orc_step(s, nCycle);
        (void)dtBefore;
        if (r < 0) break;
        if (log) {
            log[3 * a + 0] = s->maxDelta;
            log[3 * a + 1] = s->dt;
            log[3 * a + 2] = r;
        }
        a++;
    }
    return a;
}

/* ------------------------------------------------------------------------ */
/* Reductions: src/maths.cu:157-200, 294-377, 497-680 plus the residual.    */
/* Evaluated on the current B, J, detJac (call orc_refresh_fields first).   */
/* ------------------------------------------------------------------------ */

static R wedge_min_at(const orc_state* s, int i, int j, int k, int* convex) {
    const P* p = &s->p;
    int u, v, w, l;
    R wmin = 0;
    const R* x = s->xb;
    size_t gc = 3 * GI(p, i + 1, j + 1, k + 1);
    *convex = 1;
    for (u = 0; u <= 2; u += 2)
        for (v = 0; v <= 2; v += 2)
            for (w = 0; w <= 2; w += 2) {
                R d1[3], d2[3], d3[3], c[3], wc;
                size_t gu = 3 * GI(p, i + u, j + 1, k + 1), gv = 3 * GI(p, i + 1, j + v, k + 1),
                       gw = 3 * GI(p, i + 1, j + 1, k + w);
                for (l = 0; l < 3; l++) {
                    d1[l] = x[gu + l] - x[gc + l];
                    d2[l] = x[gv + l] - x[gc + l];
                    d3[l] = x[gw + l] - x[gc + l];
                }
                cross3(d1, d2, c);
                wc = dot3(c, d3);
                if ((wc < 0) && ((u + v + w == 2) || (u + v + w == 6))) *convex = -1;
                if ((wc > 0) && ((u + v + w == 0) || (u + v + w == 4))) *convex = -1;
                if (u + v + w == 0) wmin = -wc;
                if ((u + v + w == 0) || (u + v + w == 4)) wc = -wc;
                if (wc < wmin) wmin = wc;
            }
    return wmin;
}

void orc_reduce(const orc_state* s, gm_reduction* r) {
    const P* p = &s->p;
    int k;
    double B2 = 0, res = 0, resn = 0, resd = 0, Bmax = 0, Jmax = 0, jxbmax = 0, mind = 1e300, wmin = 1e300, e1 = 0, e2 = 0;
    double U2 = 0, Umax = 0;
    int convex = 1;
#pragma omp parallel for schedule(static) reduction(+ : B2, res, resn, resd, e1, e2, U2) reduction(max : Bmax, Jmax, jxbmax, Umax) reduction(min : mind, wmin, convex)
    for (k = 0; k < p->nz; k++) {
        int i, j;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                size_t g = GI(p, i + 1, j + 1, k + 1), q = II(p, i, j, k);
                const R* Bv = &s->B[3 * g];
                const R* Jv = &s->J[3 * q];
                R jxb[3], b2, q1;
                double bn, jn, cn;
                int bound, cv;
                R wm;
                cross3(Jv, Bv, jxb);
                b2 = dot3(Bv, Bv);
                q1 = RSQRT(dot3(jxb, jxb)) / b2;
                if (q1 > jxbmax) jxbmax = q1;
                bn = sqrt((double)Bv[0] * Bv[0] + (double)Bv[1] * Bv[1] + (double)Bv[2] * Bv[2]);
                jn = sqrt((double)Jv[0] * Jv[0] + (double)Jv[1] * Jv[1] + (double)Jv[2] * Jv[2]);
                {
                    double cx = (double)Jv[1] * Bv[2] - (double)Jv[2] * Bv[1];
                    double cy = (double)Jv[2] * Bv[0] - (double)Jv[0] * Bv[2];
                    double cz = (double)Jv[0] * Bv[1] - (double)Jv[1] * Bv[0];
                    cn = sqrt(cx * cx + cy * cy + cz * cz);
                }
                if (jn * bn > 0) res += cn / (jn * bn);
                resn += cn;
                resd += jn * bn;
                if (bn > Bmax) Bmax = bn;
                if (jn > Jmax) Jmax = jn;
                {
                    double e = (double)s->detJac[g];
                    if (e < mind) mind = e;
                }
                bound = (i == 0) + (j == 0) + (k == 0) + (i == p->nx - 1) + (j == p->ny - 1) + (k == p->nz - 1);
                B2 += (double)b2 * (double)s->detJac[g] / (double)(1 << bound);
                if (p->inertia) {
                    /* U2_det (maths.cu:684-710) and mag (diagnostics.cu:124-130) */
                    const R* u = &s->uu[3 * q];
                    const double un = sqrt((double)u[0] * u[0] + (double)u[1] * u[1] + (double)u[2] * u[2]);
                    U2 += (double)(dot3(u, u) * s->detJac[g]) / (double)(1 << bound);
                    if (un > Umax) Umax = un;
                }
                wm = wedge_min_at(s, i, j, k, &cv);
                if ((double)wm < wmin) wmin = wm;
                if (cv < convex) convex = cv;
                {
                    double bx = Bv[0], by = Bv[1], bz = (double)Bv[2] - 1.;
                    e1 += bx * bx + by * by + bz * bz;
                }
                {
                    double x = (double)p->dx * i + p->Ox, y = (double)p->dy * j + p->Oy, z = (double)p->dz * k + p->Oz;
                    double ph = exp(-(x * x + y * y) / ((double)p->ar * p->ar) - z * z / ((double)p->az * p->az)) * p->phi1;
                    const R* xv = &s->xb[3 * g];
                    double a0 = xv[0] - cos(ph) * x - sin(ph) * y;
                    double a1 = xv[1] + sin(ph) * x - cos(ph) * y;
                    double a2 = xv[2] - z;
                    e2 += a0 * a0 + a1 * a1 + a2 * a2;
                }
            }
    }
    /* detJac on the ghost planes of non-periodic faces (inner in-plane
     * extent); periodic ghost planes are images of inner points. */
    {
        int i, j, side;
        for (side = 0; side < 2; side++) {
            if (!p->zPeri)
                for (j = 1; j <= p->ny; j++)
                    for (i = 1; i <= p->nx; i++) {
                        double e = s->detJac[GI(p, i, j, side * (p->nz + 1))];
                        if (e < mind) mind = e;
                    }
            if (!p->yPeri)
                for (j = 1; j <= p->nz; j++)
                    for (i = 1; i <= p->nx; i++) {
                        double e = s->detJac[GI(p, i, side * (p->ny + 1), j)];
                        if (e < mind) mind = e;
                    }
            if (!p->xPeri)
                for (j = 1; j <= p->nz; j++)
                    for (i = 1; i <= p->ny; i++) {
                        double e = s->detJac[GI(p, side * (p->nx + 1), i, j)];
                        if (e < mind) mind = e;
                    }
        }
    }
    r->B2 = B2 * (double)p->dx * (double)p->dy * (double)p->dz;
    r->U2 = U2 * (double)p->dx * (double)p->dy * (double)p->dz;
    r->UMax = Umax;
    r->BMax = Bmax;
    r->JMax = Jmax;
    r->JxB_B2Max = jxbmax;
    r->residual = resd > 0 ? resn / resd : 0;
    r->residualPw = res / (double)s->N;
    r->minDetJac = mind;
    r->wedgeMin = wmin;
    r->convex = convex;
    r->errB_1ez = sqrt(e1) / sqrt((double)s->N);
    r->errXb_XbAn = sqrt(e2) / sqrt((double)s->N);
}

/* Grid-quality fields at the inner points, inner layout i + nx (j + ny k):
 * - cellVol: the signed volume of the cell towards +x, +y, +z,
 *   ((x(i+1) - x) x (x(j+1) - x)) . (x(k+1) - x)  (dirCellVol, src/maths.cu:443-493);
 * - convexity: +1, or -1 where a corner wedge has the wrong orientation
 *   (gridConvexity, src/maths.cu:573-643);
 * - wedgeMin: the smallest of the 8 corner wedge products with the sign
 *   convention of gridWedgeMin (src/maths.cu:497-569).
 * The last two come from wedge_min_at, which the reductions also use.  Any
 * output pointer may be NULL. */
void orc_grid_fields(const orc_state* s, R* cellVol, R* convexity, R* wedgeMin) {
    const P* p = &s->p;
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < p->nz; k++) {
        int i, j, l;
        for (j = 0; j < p->ny; j++)
            for (i = 0; i < p->nx; i++) {
                const size_t q = II(p, i, j, k);
                const R* x = s->xb;
                const size_t gc = 3 * GI(p, i + 1, j + 1, k + 1);
                if (cellVol) {
                    R d1[3], d2[3], d3[3], c[3];
                    const size_t g1 = 3 * GI(p, i + 2, j + 1, k + 1), g2 = 3 * GI(p, i + 1, j + 2, k + 1),
                                 g3 = 3 * GI(p, i + 1, j + 1, k + 2);
                    for (l = 0; l < 3; l++) {
                        d1[l] = x[g1 + l] - x[gc + l];
                        d2[l] = x[g2 + l] - x[gc + l];
                        d3[l] = x[g3 + l] - x[gc + l];
                    }
                    cross3(d1, d2, c);
                    cellVol[q] = dot3(c, d3);
                }
                if (convexity || wedgeMin) {
                    int cv;
                    const R wm = wedge_min_at(s, i, j, k, &cv);
                    if (convexity) convexity[q] = (R)cv;
                    if (wedgeMin) wedgeMin[q] = wm;
                }
            }
    }
}

/* The force-free parameter eps* (src/maths.cu:203-290, driven by
 * src/diagnostics.cu:32-47): along the central column i = nx/2, j = ny/2,
 * a_k = (J.B)/(B.B) in REAL (JB_B2) and z_k the grid's z coordinate; eps* is
 * the largest sqrt(2) |(a_n - a_p) / (z_n - z_p)| over the pairs with
 * z_n != z_p (0 for the others), the product formed in double and stored in
 * REAL, then findDevMax over the nz x nz values (NaN never wins,
 * src/maths.cu:58-97).  The reference's kernel covers every pair when
 * nz <= 256 or nz is a multiple of 256, its block size; for other nz its
 * second block reads shared memory that no thread wrote, and all pairs are
 * taken here. */
double orc_eps_star(const orc_state* s) {
    const P* p = &s->p;
    const int i = p->nx / 2, j = p->ny / 2, nz = p->nz;
    R* a = (R*)malloc(sizeof(R) * (size_t)nz);
    R* z = (R*)malloc(sizeof(R) * (size_t)nz);
    R m = 0;
    int n, q;
    if (!a || !z) {
        free(a);
        free(z);
        return NAN;
    }
    for (n = 0; n < nz; n++) {
        const size_t g = GI(p, i + 1, j + 1, n + 1), l = II(p, i, j, n);
        const R* Bv = &s->B[3 * g];
        const R* Jv = &s->J[3 * l];
        a[n] = dot3(Jv, Bv) / dot3(Bv, Bv);
        z[n] = s->xb[3 * g + 2];
    }
    for (q = 0; q < nz; q++)
        for (n = 0; n < nz; n++) {
            R v = 0;
            if (z[n] != z[q]) v = (R)(1.414213562373095 * (double)RABS((a[n] - a[q]) / (z[n] - z[q])));
            if (v > m) m = v;
        }
    free(a);
    free(z);
    return (double)m;
}

int orc_real_bits(void) { return ORC_BITS; }
