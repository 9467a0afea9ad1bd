// gm_stage_tma.cuh -- the RK stage kernel with TMA-fed plane rings.
//
// Same arithmetic as k_stage (gm_kernels_impl.cuh); different data movement:
//   * tiles are 32 x 8 columns (compile time), one warp per tile row;
//   * one thread streams, plane by plane, every operand of the stage with
//     cp.async.bulk.tensor into shared-memory rings: the grid positions
//     (tile + 2-point halo, all three components as one 4-D box), the scaled
//     field B0s (same box) and the increments k_0..k_{n-1} over the tile;
//     completion is tracked by one mbarrier per ring slot;
//   * J for plane k is formed in the same iteration as B of plane k+1, so an
//     iteration needs a single __syncthreads;
//   * every shared-memory access is a constant offset from a per-plane base.
// Waits on the mbarriers are bounded: after kWaitLimit polls the CTA records
// GM_ST_TIMEOUT, drains the copies it has in flight (again bounded) and
// returns.
#pragma once

#include <cuda.h>

#include "gm_kernels_impl.cuh"

namespace gmk {

constexpr int TY2 = 8;                   // warps per CTA (one tile row each, per row group)
constexpr int HX2 = TX + 4;              // position-plane row: the tile + 2-point halo
constexpr int BX2 = TX + 2;              // B-plane row: the tile + face halo
// resident CTAs per SM the stage kernel is compiled for (register budget)
#ifndef GM_STAGE_MINB
#define GM_STAGE_MINB 3
#endif
constexpr unsigned kWaitLimit = 1u << 22;

// Tile of R row groups: 32 x 8R columns, each thread owning the points of
// rows ty, ty + 8, ..., ty + 8 (R - 1) of its column.
template <int R>
struct TileShape {
    static constexpr int TYR = TY2 * R;                  // tile rows
    static constexpr int HYR = TYR + 4, BYR = TYR + 2;   // position / B plane rows
    static constexpr int PLANE_C = HYR * HX2;            // elements of one component of a position plane
    static constexpr int PLANE_X = 3 * PLANE_C;
};

// Stride of a position-plane slot in elements: the plane rounded up so every
// slot (a TMA destination) starts on a 128-byte boundary.
template <typename T, int R>
constexpr int slot_elems() {
    return (int)(((TileShape<R>::PLANE_X * sizeof(T) + 127) / 128) * 128 / sizeof(T));
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait; returns false when the limit ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (unsigned it = 0; it < kWaitLimit; it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}


// Reciprocal for the stage kernel: FP32 uses the hardware approximation plus
// one Newton step (within ~1 ulp; FP32 parity is judged at 1e-5), FP64 the
// correctly rounded one.
__device__ __forceinline__ float rcp_stage(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return fmaf(fmaf(-x, r, 1.0f), r, r);
}
__device__ __forceinline__ double rcp_stage(double x) { return __drcp_rn(x); }

// det(a, b, c) of the columns of A.  In FP32 the determinant of a strongly
// sheared cell (|det| small against the bound |a|_1 |b|_1 |c|_1 of the six
// Sarrus products) is recomputed in double from the same entries.
template <typename T>
__device__ __forceinline__ T det_cols(const T A[3][3]) {
    T d = det3(A);
    if (sizeof(T) == 4) {
        const T m = (fabs(A[0][0]) + fabs(A[1][0]) + fabs(A[2][0])) * (fabs(A[0][1]) + fabs(A[1][1]) + fabs(A[2][1])) *
                    (fabs(A[0][2]) + fabs(A[1][2]) + fabs(A[2][2]));
        if (fabs(d) < (T)0.03125 * m) {
            double jd[3][3];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) jd[r][c] = (double)A[r][c];
            d = (T)det3<double>(jd);
        }
    }
    return d;
}

// B at a non-face point from the position planes (constant offsets), in the
// form B = (s_x a + s_y b + s_z c) / det(a, b, c) with the unscaled central
// differences a = x(+x) - x(-x), b, c and the pre-scaled field
// s = (4 dy dz B0x, 4 dx dz B0y, 4 dx dy B0z): since jac = [a/2dx, b/2dy,
// c/2dz], this is jac.B0 / det(jac) of B_JacB0 (rungeKutta.cu:79-99) with
// the constant factors folded.  x and s come from shared-memory planes at the
// same offset o; PC is the component stride of a plane.  Returns the columns
// a, b, c in Am[l][0..2] and 1/det(a, b, c) in *rdet (Delta = 1 / (8 dx dy dz
// rdet)).
template <typename T, int PC>
__device__ __forceinline__ void b_point(const T* __restrict__ xm, const T* __restrict__ x0, const T* __restrict__ xp,
                                        int o, const T* __restrict__ b0s, T Bv[3], T Am[3][3], T* rdet) {
    const T s0 = b0s[o], s1 = b0s[o + PC], s2 = b0s[o + 2 * PC];
#pragma unroll
    for (int l = 0; l < 3; l++) {
        const int q = o + l * PC;
        Am[l][0] = x0[q + 1] - x0[q - 1];
        Am[l][1] = x0[q + HX2] - x0[q - HX2];
        Am[l][2] = xp[q] - xm[q];
    }
    const T r = rcp_stage(det_cols(Am));
#pragma unroll
    for (int l = 0; l < 3; l++) Bv[l] = (Am[l][0] * s0 + Am[l][1] * s1 + Am[l][2] * s2) * r;
    *rdet = r;
}

// One B point in a shared-memory B plane: three components and a pad, so a
// neighbour is one 128-bit load (two for double).
__device__ __forceinline__ void st_b(float* d, const float v[3]) {
    *reinterpret_cast<float4*>(d) = make_float4(v[0], v[1], v[2], 0.f);
}
__device__ __forceinline__ void st_b(double* d, const double v[3]) {
    reinterpret_cast<double2*>(d)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(d)[1] = make_double2(v[2], 0.0);
}
__device__ __forceinline__ void ld_b(const float* d, float v[3]) {
    const float4 q = *reinterpret_cast<const float4*>(d);
    v[0] = q.x; v[1] = q.y; v[2] = q.z;
}
__device__ __forceinline__ void ld_b(const double* d, double v[3]) {
    const double2 q0 = reinterpret_cast<const double2*>(d)[0], q1 = reinterpret_cast<const double2*>(d)[1];
    v[0] = q0.x; v[1] = q0.y; v[2] = q1.x;
}

// Shared memory of the stage kernels, all in the dynamic buffer (the base is
// rounded up to 128 bytes at run time; the launch asks for 128 bytes of
// slack):
//   XR position-plane slots (the tile + 2-point halo, three components),
//   2 slots of B0s planes (same box),
//   2 slots of k-planes (the n arrays k_0..k_{n-1} over the tile; 1 slot in
//   the late stages, so that the CTAs per SM the kernel is built for fit),
//   2 B planes (float4 per point: B and a pad),
//   XR + 4 mbarriers, warp maxima, the abort flag and the work-item slot.
// Every slot is a multiple of 128 bytes, the alignment TMA destinations need.
template <typename T, bool PRESS, int NS, int R>
struct StageSmem {
    static constexpr int XR = PRESS ? 5 : 4;                      // position ring (one plane of prefetch)
    static constexpr int SLOT = slot_elems<T, R>();
    static constexpr int NK = NS;                                 // k arrays read by stage NS
    static constexpr int KBOX = 3 * TileShape<R>::TYR * TX;       // elements of one k-array plane
    static constexpr int KSLOT = NK * KBOX;
    // k-plane slots: two (the next plane streams in while this one is read),
    // or one where two would not leave room for the CTAs per SM the kernel is
    // built for (its plane is then loaded during the B phase of the same
    // iteration, behind a second barrier)
    static constexpr int KS = R == 1 ? ((PRESS && NS == 5) ? 1 : 2) : ((NS >= 4 || (PRESS && NS >= 3)) ? 1 : 2);
    static constexpr int PLANE_B = 4 * TileShape<R>::BYR * BX2;
    static constexpr size_t OFF_B0 = sizeof(T) * (size_t)XR * SLOT;
    static constexpr size_t OFF_K = OFF_B0 + sizeof(T) * 2 * (size_t)SLOT;
    static constexpr size_t OFF_B = OFF_K + sizeof(T) * KS * (size_t)KSLOT;
    static constexpr size_t OFF_BAR = OFF_B + sizeof(T) * 2 * (size_t)PLANE_B;
    static constexpr int NBAR = XR + 2 + KS;                     // x slots, 2 B0s slots, k slots
    static constexpr size_t OFF_WMAX = OFF_BAR + 8 * NBAR;
    static constexpr size_t OFF_CTL = OFF_WMAX + 16 * TY2;
    static constexpr size_t BYTES = 128 + OFF_CTL + 64;
};

// Copy bookkeeping of a CTA, kept in shared memory and touched by the
// producer thread only (abort and the work item are read by all threads after
// a barrier).
struct StageCtl {
    uint32_t ph;                 // next completion parity of each mbarrier
    int x_iss, x_done;           // position planes issued / completed
    int b_iss, b_done;           // B0s planes
    int k_iss, k_done;           // k planes
    int abort;                   // a bounded wait ran out
    int work;                    // batched launch: the current work item
};

// Kind of a B-region point, fixed for the whole z march of a thread.
enum { BK_SKIP = 0, BK_INNER = 1, BK_FACE_X = 2, BK_FACE_Y = 3 };

// One RK stage over the 32 x 8R x TZ block (bx, by, bz) of one case.
// Iteration kk of the z march computes B on plane kb = kk - 1 (the tile and
// its face halo) and then J, k_n and the stage position on plane kc = kk - 2.
// Each thread keeps, for each of its R points of the plane, B at kc - 1, kc,
// kc + 1 and the
// diagonals a, b, c and 1/det of plane kc in registers, so J needs only the
// four in-plane neighbours' B from shared memory, written in the previous
// iteration.  Operands arrive by TMA one iteration ahead: position plane
// kk + 1 (into the slot of plane kk + 1 - XR: the B phase last read it in the
// previous iteration, and so did the pressure gradient, which reads planes
// kc - 1 .. kc + 1, with its fifth slot), the B0s plane of the next B phase
// and the k planes of the next J phase.  `base` is the 128-byte aligned shared buffer
// with initialised mbarriers; the mbarrier parities in its StageCtl carry
// over to the next tile.  Returns false
// after a bounded wait ran out or an alignment check failed (the status word
// says which).
template <typename T, bool PRESS, int NS, int R>
__device__ __forceinline__ bool stage_tile(const StageArgsTMA<T>& A, int bx, int by, int bz, unsigned char* base) {
    using L = StageSmem<T, PRESS, NS, R>;
    using S = TileShape<R>;
    constexpr bool LAST = NS == 5;
    constexpr int n = NS;
    constexpr int XR = L::XR;
    constexpr int SLOT = L::SLOT;
    constexpr int PLANE_B = L::PLANE_B;
    constexpr int TYR = S::TYR, BYR = S::BYR, PC = S::PLANE_C;

    const StageArgs<T>& a = A.a;
    const KP<T>& p = a.p;
    DevState* st = a.st;
    // a stopped run, or an earlier stage of this step that gave up a wait or
    // failed its alignment check: nothing to compute
    if (st->done || (st->status & (GM_ST_TIMEOUT | GM_ST_ALIGN))) return true;

    T* xs = reinterpret_cast<T*>(base);                                   // XR position slots
    T* b0r = reinterpret_cast<T*>(base + L::OFF_B0);                       // 2 B0s slots
    T* kr = reinterpret_cast<T*>(base + L::OFF_K);                         // k slots
    T* bs = reinterpret_cast<T*>(base + L::OFF_B);                         // 2 B planes
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + L::OFF_BAR);       // x | B0s | k
    T* s_wmax = reinterpret_cast<T*>(base + L::OFF_WMAX);
    StageCtl* ctl = reinterpret_cast<StageCtl*>(base + L::OFF_CTL);
    int* s_abort = &ctl->abort;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    // the producer (copy issue and waits) is lane 0 of the last warp, which
    // computes no face-halo B points
    const bool producer = tid == (TY2 - 1) * TX;
    const int i0 = bx * TX, j0 = by * TYR, k0 = bz * a.TZ;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int kend = min(k0 + a.TZ, nz);
    const int cur = st->cur;
    const int mapi = (n == 0) ? cur : 2 + ((n - 1) & 1);
    const CUtensorMap* tmap = &A.tm[mapi];
    const CUtensorMap* tmb0 = &A.tm[4];
    const T dtT = (T)st->dt;
    const int KC = (int)p.kcs;
    const int cs = (int)p.cs;
    const int pxy = p.px * p.py;
    const bool zPeri = p.zPeri != 0;
    constexpr uint32_t kPlaneBytes = S::PLANE_X * sizeof(T);
    constexpr uint32_t kKBytes = (uint32_t)(L::KSLOT * sizeof(T));

    // self-check of the alignment TMA needs: destination slots on 128 bytes,
    // mbarriers on 8 bytes, tensor maps on 64 bytes, box start on 16 bytes; on
    // failure record a status bit and issue no copy
    if ((smem_u32(xs) & 127u) || (smem_u32(b0r) & 127u) || (smem_u32(kr) & 127u) || (smem_u32(bs) & 15u) ||
        (smem_u32(bars) & 7u) || (reinterpret_cast<uintptr_t>(&A.tm[0]) & 63u) || ((i0 * (int)sizeof(T)) & 15)) {
        if (producer) atomicOr(&st->status, (unsigned)GM_ST_ALIGN);
        return false;
    }

    // ---- per-thread descriptors, fixed for the whole z march ----------------
    // the thread's own points: column i0 + tx, rows ty + 8 r (r < R)
    const int ic = i0 + tx;
    int jc[R], ox1[R], ob1[R], tyx[R], kind1[R], gxy1[R], lin0[R];
    bool own[R], img_xy[R];
    T exy[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int tyr = ty + TY2 * r;
        jc[r] = j0 + tyr;
        own[r] = ic < nx && jc[r] < ny;
        ox1[r] = (tyr + 2) * HX2 + (tx + 2);           // in a position / B0s plane
        ob1[r] = 4 * ((tyr + 1) * BX2 + (tx + 1));     // in a B plane
        tyx[r] = tyr * TX + tx;                        // in a k plane
        // in a partial tile the ghost column i = nx or row j = ny is a tile point
        kind1[r] = BK_SKIP;
        const bool xo1 = ic >= nx, yo1 = jc[r] >= ny;
        if (ic <= nx && jc[r] <= ny && !(xo1 && yo1)) {
            if (xo1 && !p.xPeri) kind1[r] = BK_FACE_X;
            else if (yo1 && !p.yPeri) kind1[r] = BK_FACE_Y;
            else kind1[r] = BK_INNER;
        }
        exy[r] = own[r] ? p.ex[ic] * p.ey[jc[r]] : (T)0;
        gxy1[r] = (ic + 2) + p.px * (jc[r] + 2);      // padded offset without the plane term
        lin0[r] = ic + p.kpx * jc[r];                 // k_m index of the own column
        img_xy[r] = (p.xPeri && (ic < 2 || ic >= nx - 2)) || (p.yPeri && (jc[r] < 2 || jc[r] >= ny - 2));
    }
    // one face-halo point for warps 0-2: the rows above and below the tile
    // (warps 0 and 1) and its left and right columns (warp 2, 2 TYR <= 32 points)
    int jj2 = 0, ii2 = 0, kind2 = BK_SKIP;
    if (ty == 0) { jj2 = 0; ii2 = tx + 1; }
    else if (ty == 1) { jj2 = BYR - 1; ii2 = tx + 1; }
    else if (ty == 2 && tx < 2 * TYR) { jj2 = (tx % TYR) + 1; ii2 = tx < TYR ? 0 : BX2 - 1; }
    else ii2 = -1;
    const int i2 = i0 - 1 + ii2, j2 = j0 - 1 + jj2;
    if (ii2 >= 0 && i2 <= nx && j2 <= ny) {
        const bool xo2 = (i2 < 0 || i2 >= nx);
        const bool yo2 = (j2 < 0 || j2 >= ny);
        if (xo2 && yo2) kind2 = BK_SKIP;
        else if (xo2 && !p.xPeri) kind2 = BK_FACE_X;
        else if (yo2 && !p.yPeri) kind2 = BK_FACE_Y;
        else kind2 = BK_INNER;
    }
    const int ox2 = (jj2 + 1) * HX2 + (ii2 + 1);
    const int ob2 = 4 * (jj2 * BX2 + ii2);
    const int kplane = p.kpx * ny;
    const T* __restrict__ ezp = p.ez;

    auto xslot = [&](int plane) { return (plane + 20) % XR; };
    // thread 0: wait for the copy tracked by mbarrier b, then flip its parity
    auto wait_bar = [&](int b) {
        const bool ok = mbar_wait_bounded(&bars[b], (ctl->ph >> b) & 1u);
        ctl->ph ^= 1u << b;
        return ok;
    };
    auto issue_x = [&](int q) {
        uint64_t* b = &bars[xslot(q)];
        mbar_expect_tx(b, kPlaneBytes);
        tma_load_4d(xs + xslot(q) * SLOT, tmap, b, i0, j0, q + 2, 0);
    };
    auto issue_b0 = [&](int q) {
        uint64_t* b = &bars[XR + (q & 1)];
        mbar_expect_tx(b, kPlaneBytes);
        tma_load_4d(b0r + (q & 1) * SLOT, tmb0, b, i0, j0, q + 2, 0);
    };
    constexpr int KS = L::KS;
    auto kbar = [&](int q) { return XR + 2 + (KS == 2 ? (q & 1) : 0); };
    auto kslot = [&](int q) { return kr + (KS == 2 ? (q & 1) : 0) * L::KSLOT; };
    auto issue_k = [&](int q) {
        uint64_t* b = &bars[kbar(q)];
        mbar_expect_tx(b, kKBytes);
#pragma unroll
        for (int m = 0; m < n; m++)
            tma_load_4d(kslot(q) + m * L::KBOX, &A.tm[5 + m], b, i0, j0, q, 0);
    };
    // ring positions relative to plane kk, from one modulo per iteration
    auto xring = [&](int m, int back) { int s = m - back; s += s < 0 ? XR : 0; return xs + s * SLOT; };
    // the face formula at x / y face points (no initial-distortion terms: those
    // concern the z faces only) and at the z ghost planes
    auto face_b = [&](int face, int i, int j, int kb, T Bv[3]) {
        Tile<T, 4, XR, 20> tl;
        tl.xs = xs;
        tl.i0 = i0; tl.j0 = j0; tl.HX = HX2; tl.HY = S::HYR;
        tl.slot = SLOT;
        T D;
        b_face<T, false>(p, tl, a.B0, face, i, j, kb, Bv, &D);
    };
    auto face_bz = [&](int i, int j, int kb, T Bv[3]) {
        Tile<T, 4, XR, 20> tl;
        tl.xs = xs;
        tl.i0 = i0; tl.j0 = j0; tl.HX = HX2; tl.HY = S::HYR;
        tl.slot = SLOT;
        T D;
        b_face<T, true>(p, tl, a.B0, 2, i, j, kb, Bv, &D);
    };

    // copies issued / completed so far (the producer): position planes
    // k0-2 .. kend+1, B0s planes k0-1 .. kend, k planes k0 .. kend-1
    if (producer) {
        // failure-detection test (a.stall): the first position planes are
        // withheld, so the bounded waits for them run out
        if (!a.stall)
            for (int q = k0 - 2; q <= min(k0 + 1, kend + 1); q++) issue_x(q);
        ctl->x_iss = min(k0 + 1, kend + 1);
        ctl->x_done = k0 - 3;
        issue_b0(k0 - 1);
        ctl->b_iss = k0 - 1;
        ctl->b_done = k0 - 2;
        ctl->k_iss = k0 - 1;
        ctl->k_done = k0 - 1;
    }

    T dmax = 0;
    bool bad = false;
    // own columns: B at kc-1, kc, kc+1 and a, b, c, 1/det at kc
    T Bm[R][3], Bz[R][3], Bp[R][3], Ac[R][3][3], An[R][3][3], Rc[R], Rn[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
#pragma unroll
        for (int l = 0; l < 3; l++) {
            Bm[r][l] = 0; Bz[r][l] = 0; Bp[r][l] = 0;
            Ac[r][l][0] = 0; Ac[r][l][1] = 0; Ac[r][l][2] = 0;
            An[r][l][0] = 0; An[r][l][1] = 0; An[r][l][2] = 0;
        }
        Rc[r] = 0; Rn[r] = 0;
    }

    for (int kk = k0; kk <= kend + 1; kk++) {
        // (1) the producer waits for position plane kk, the B0s plane of
        // kb = kk-1 and the k planes of kc = kk-2
        if (producer) {
            const int need = min(kk, kend + 1);
            bool ok = true;
            while (ok && ctl->x_done < need) { ok = wait_bar(xslot(ctl->x_done + 1)); ctl->x_done++; }
            while (ok && ctl->b_done < kk - 1) { ok = wait_bar(XR + ((ctl->b_done + 1) & 1)); ctl->b_done++; }
            if (n > 0 && KS == 2)
                while (ok && ctl->k_done < kk - 2) { ok = wait_bar(kbar(ctl->k_done + 1)); ctl->k_done++; }
            if (!ok) {
                *s_abort = 1;
                atomicOr(&st->status, (unsigned)GM_ST_TIMEOUT);
            }
        }
        __syncthreads();
        if (*s_abort) break;
        // (2) refills, into slots whose last reader was the previous iteration
        // (every thread is past this iteration's barrier)
        if (producer) {
            const int qx = kk + 1;
            if (qx <= kend + 1 && qx > ctl->x_iss) { issue_x(qx); ctl->x_iss = qx; }
            if (kk <= kend && kk > ctl->b_iss) { issue_b0(kk); ctl->b_iss = kk; }
            // k planes: the next J phase's (two slots), or this one's (one slot:
            // the previous J phase, its last reader, is behind the barrier)
            const int qk = KS == 2 ? kk - 1 : kk - 2;
            if (n > 0 && qk >= k0 && qk < kend && qk > ctl->k_iss) { issue_k(qk); ctl->k_iss = qk; }
        }
        const int mx = (kk + 20) % XR;      // ring slot of position plane kk
        // (3) B on plane kb = kk - 1 into B plane kb & 1
        const int kb = kk - 1;
        T Bv[R][3];
        {
            T* bdst = bs + (kb & 1) * PLANE_B;
            const T* xm = xring(mx, 2);
            const T* x0 = xring(mx, 1);
            const T* xq = xring(mx, 0);
            const T* s0 = b0r + (kb & 1) * SLOT;
            const bool zo = (kb < 0 || kb >= nz);
#pragma unroll
            for (int r = 0; r < R; r++) {
                Bv[r][0] = 0; Bv[r][1] = 0; Bv[r][2] = 0;
                if (!zo) {
                    if (kind1[r] != BK_SKIP) {
                        if (kind1[r] == BK_INNER) b_point<T, PC>(xm, x0, xq, ox1[r], s0, Bv[r], An[r], &Rn[r]);
                        else face_b(kind1[r] == BK_FACE_X ? 0 : 1, ic, jc[r], kb, Bv[r]);
                        st_b(bdst + ob1[r], Bv[r]);
                    }
                } else if (!zPeri) {
                    // line-tied ghost plane: only the own columns are needed
                    if (own[r]) face_bz(ic, jc[r], kb, Bv[r]);
                } else {
                    // periodic image plane: only the own columns are needed
                    if (own[r]) b_point<T, PC>(xm, x0, xq, ox1[r], s0, Bv[r], An[r], &Rn[r]);
                }
            }
            if (!zo && kind2 != BK_SKIP) {
                T Bh[3], Ah[3][3], Rh;
                if (kind2 == BK_INNER) b_point<T, PC>(xm, x0, xq, ox2, s0, Bh, Ah, &Rh);
                else face_b(kind2 == BK_FACE_X ? 0 : 1, i2, j2, kb, Bh);
                st_b(bdst + ob2, Bh);
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int l = 0; l < 3; l++) { Bm[r][l] = Bz[r][l]; Bz[r][l] = Bp[r][l]; Bp[r][l] = Bv[r][l]; }
        // (4) J, k_n and the stage position on plane kc = kk - 2
        const int kc = kk - 2;
        if (KS == 1 && kc >= k0) {
            // one k slot: the producer waits for this plane's k copies (issued
            // at the top of this iteration), then a barrier publishes them
            if (producer) {
                bool ok = true;
                while (ok && ctl->k_done < kc) { ok = wait_bar(kbar(ctl->k_done + 1)); ctl->k_done++; }
                if (!ok) {
                    *s_abort = 1;
                    atomicOr(&st->status, (unsigned)GM_ST_TIMEOUT);
                }
            }
            __syncthreads();
            if (*s_abort) break;
        }
        if (kc >= k0) {
            const T* bc = bs + (kc & 1) * PLANE_B;
            const T* x0 = xring(mx, 2);   // position plane kc
            const T ezk = __ldg(&ezp[kc]);
            const bool zimg = zPeri && (kc < 2 || kc >= nz - 2);
#pragma unroll
            for (int r = 0; r < R; r++) {
                if (!own[r]) continue;
                // in-plane neighbours' B: -x, +x, -y, +y
                T bxm[3], bxp[3], bym[3], byp[3];
                ld_b(bc + ob1[r] - 4, bxm);
                ld_b(bc + ob1[r] + 4, bxp);
                ld_b(bc + ob1[r] - 4 * BX2, bym);
                ld_b(bc + ob1[r] + 4 * BX2, byp);
                // Stokes current (current.cu:290-406).  The circulation around a
                // quadrilateral P1..P4, sum (B_a + B_b).(x_b - x_a) over its edges,
                // regroups exactly into sum B_a.(x_{a+1} - x_{a-1}); for the quads
                // through the face neighbours (-x,-y,+x,+y), (-y,-z,+y,+z) and
                // (-z,-x,+z,+x) that is I0 = b.dxB - a.dyB, I1 = c.dyB - b.dzB and
                // I2 = a.dzB - c.dxB with the diagonals a = x(+x) - x(-x), b, c and
                // dxB = B(+x) - B(-x), ...  The quads' area vectors are
                // (1/2) a x b, (1/2) b x c, (1/2) c x a (for a quadrilateral,
                // (1/4) sum of consecutive edge cross products = (1/2) d1 x d2),
                // and the matrix with those rows has the inverse
                // 2 [a b c] P / det(a, b, c), so J = (a I1 + b I2 + c I0) / det.
                T I0 = 0, I1 = 0, I2 = 0;
#pragma unroll
                for (int l = 0; l < 3; l++) {
                    const T dx = bxp[l] - bxm[l], dy = byp[l] - bym[l], dz = Bp[r][l] - Bm[r][l];
                    I0 += Ac[r][l][1] * dx - Ac[r][l][0] * dy;
                    I1 += Ac[r][l][2] * dy - Ac[r][l][1] * dz;
                    I2 += Ac[r][l][0] * dz - Ac[r][l][2] * dx;
                }
                T Jv[3];
#pragma unroll
                for (int l = 0; l < 3; l++) Jv[l] = (Ac[r][l][0] * I1 + Ac[r][l][1] * I2 + Ac[r][l][2] * I0) * Rc[r];
                const int lin = lin0[r] + kplane * kc;
                T kn[3];
                cross3(Jv, Bz[r], kn);
                const T f = dtT * (exy[r] * ezk);
#pragma unroll
                for (int l = 0; l < 3; l++) kn[l] *= f;
                if (PRESS) {
                    Tile<T, 4, XR, 20> tl;
                    tl.xs = xs;
                    tl.i0 = i0; tl.j0 = j0; tl.HX = HX2; tl.HY = S::HYR;
                    tl.slot = SLOT;
                    T gp[3];
                    const T D = rcp_stage(Rc[r]) * p.inv8dxdydz;     // Delta = det(a, b, c) / (8 dx dy dz)
                    grad_p<T>(p, tl, ic, jc[r], kc, D, gp);
#pragma unroll
                    for (int l = 0; l < 3; l++) kn[l] += -dtT * gp[l];
                }
                T xa[3];
#pragma unroll
                for (int l = 0; l < 3; l++) xa[l] = x0[ox1[r] + l * PC];
                const bool images = img_xy[r] || zimg;
                const int g = gxy1[r] + pxy * (kc + 2);
                const T* kp = kslot(kc) + tyx[r];    // k_m component l at kp[(3m + l) * TX * TYR]
                if (!LAST) {
                    // x_{n+1} = x_n + sum_{m<=n} (b[n+1][m] - b[n][m]) k_m (rungeKutta.cu:216-227)
#pragma unroll
                    for (int m = 0; m < n; m++) {
                        const T w = p.db[n][m];
#pragma unroll
                        for (int l = 0; l < 3; l++) xa[l] += w * kp[(3 * m + l) * TX * TYR];
                    }
                    const T w = p.db[n][n];
#pragma unroll
                    for (int l = 0; l < 3; l++) xa[l] += w * kn[l];
                    T* Kn = a.K[n];
                    Kn[lin] = kn[0];
                    Kn[KC + lin] = kn[1];
                    Kn[2 * KC + lin] = kn[2];
                    T* Xo = a.XS[n & 1];
                    if (images) {
                        store_pos<T>(p, Xo, ic, jc[r], kc, xa);
                    } else {
                        Xo[g] = xa[0];
                        Xo[cs + g] = xa[1];
                        Xo[2 * cs + g] = xa[2];
                    }
                } else {
                    // stage 5: x_6, x_new, x* and the error norm (rungeKutta.cu:251-339)
                    T km[6][3];
#pragma unroll
                    for (int m = 0; m < 5; m++)
#pragma unroll
                        for (int l = 0; l < 3; l++) km[m][l] = kp[(3 * m + l) * TX * TYR];
#pragma unroll
                    for (int l = 0; l < 3; l++) km[5][l] = kn[l];
#pragma unroll
                    for (int m = 0; m < 6; m++)
#pragma unroll
                        for (int l = 0; l < 3; l++) xa[l] += p.db[5][m] * km[m][l];
                    T xnew[3];
#pragma unroll
                    for (int l = 0; l < 3; l++) {
                        xnew[l] = xa[l];
                        T xst = xa[l];
                        T dl = 0;
                        if (l < 2 || p.zUpdate) {
                            if (p.errMode == 0) {
#pragma unroll
                                for (int m = 0; m < 6; m++) {
                                    xnew[l] += p.c[m] * km[m][l];
                                    xst += p.cst[m] * km[m][l];
                                }
                                dl = fabs(xnew[l] - xst);
                            } else {
                                // sum (c - c*) k: no cancellation against x
                                T e = 0;
#pragma unroll
                                for (int m = 0; m < 6; m++) {
                                    xnew[l] += p.c[m] * km[m][l];
                                    e += p.cmcT[m] * km[m][l];
                                }
                                dl = fabs(e);
                            }
                        }
                        if (dl > dmax) dmax = dl;     // NaN never wins (maths.cu:144-153)
                        if (!isfinite(dl) || !isfinite(xnew[l])) bad = true;   // NaN/Inf anywhere in k_0..k_5
                    }
                    if (images) {
                        store_pos<T>(p, a.X[cur], ic, jc[r], kc, xa);
                        store_pos<T>(p, a.X[cur ^ 1], ic, jc[r], kc, xnew);
                    } else {
                        T* X6 = a.X[cur];
                        T* Xn = a.X[cur ^ 1];
                        X6[g] = xa[0]; X6[cs + g] = xa[1]; X6[2 * cs + g] = xa[2];
                        Xn[g] = xnew[0]; Xn[cs + g] = xnew[1]; Xn[2 * cs + g] = xnew[2];
                    }
                }
            }
        }
        // the diagonals of plane kb become those of the next iteration's kc
#pragma unroll
        for (int r = 0; r < R; r++) {
#pragma unroll
            for (int l = 0; l < 3; l++) {
                Ac[r][l][0] = An[r][l][0]; Ac[r][l][1] = An[r][l][1]; Ac[r][l][2] = An[r][l][2];
            }
            Rc[r] = Rn[r];
        }
    }
    // drain copies still in flight (after an abort), bounded
    if (producer && *s_abort) {
        for (int q = ctl->x_done + 1; q <= ctl->x_iss; q++) wait_bar(xslot(q));
        for (int q = ctl->b_done + 1; q <= ctl->b_iss; q++) wait_bar(XR + (q & 1));
        if (n > 0)
            for (int q = ctl->k_done + 1; q <= ctl->k_iss; q++) wait_bar(kbar(q));
    }
    if (bad) atomicOr(&st->status, (unsigned)GM_ST_NAN);
    if (LAST) {
        for (int o = 16; o > 0; o >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        if (tx == 0) s_wmax[ty] = dmax;
        __syncthreads();
        if (tid == 0) {
            T m = 0;
            for (int w = 0; w < TY2; w++) m = fmax(m, s_wmax[w]);
            if (m > 0) atomicMax(&st->maxDeltaBits, (unsigned long long)__double_as_longlong((double)m));
        }
    }
    return *s_abort == 0;
}

// Shared-memory set-up common to the stage kernels: the 128-byte aligned
// base, the mbarriers and the abort flag.
template <typename T, bool PRESS, int NS, int R>
__device__ __forceinline__ unsigned char* stage_smem_setup(unsigned char* smraw) {
    using L = StageSmem<T, PRESS, NS, R>;
    unsigned char* base = smraw + ((128u - (smem_u32(smraw) & 127u)) & 127u);
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + L::OFF_BAR);
    StageCtl* ctl = reinterpret_cast<StageCtl*>(base + L::OFF_CTL);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        ctl->ph = 0;
        ctl->abort = 0;
        for (int s = 0; s < L::NBAR; s++) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    return base;
}

// One RK stage of one case: one CTA per 32 x 8R x TZ block, R =
// stage_rows<T, PRESS>() (minimum CTAs per SM: 3 for one FP32 row group, 2 for
// two, 2 in FP64).
template <typename T, bool PRESS, int NS>
__global__ void __launch_bounds__(TX * TY2, sizeof(T) == 4 ? (stage_rows<T, PRESS>() == 1 ? GM_STAGE_MINB : 2) : 2)
    k_stage_tma(const __grid_constant__ StageArgsTMA<T> A) {
    extern __shared__ __align__(128) unsigned char smraw[];
    if (A.a.st->done || (A.a.st->status & (GM_ST_TIMEOUT | GM_ST_ALIGN))) return;
    constexpr int R = stage_rows<T, PRESS>();
    unsigned char* base = stage_smem_setup<T, PRESS, NS, R>(smraw);
    stage_tile<T, PRESS, NS, R>(A, blockIdx.x, blockIdx.y, blockIdx.z, base);
}

// One RK stage of many cases: a persistent launch whose CTAs take work items
// (case, tile) from a counter until none is left; cases whose controller has
// stopped are skipped.  The counter is reset by the batched controller.
template <typename T, bool PRESS, int NS>
__global__ void __launch_bounds__(TX * TY2, 2)
    k_stage_tma_batch(const StageArgsTMA<T>* __restrict__ cases, const int4* __restrict__ work, int nwork,
                      int* __restrict__ counter) {
    using L = StageSmem<T, PRESS, NS, 1>;
    extern __shared__ __align__(128) unsigned char smraw[];
    unsigned char* base = stage_smem_setup<T, PRESS, NS, 1>(smraw);
    int* s_w = &reinterpret_cast<StageCtl*>(base + L::OFF_CTL)->work;
    for (;;) {
        if (threadIdx.x == 0 && threadIdx.y == 0) *s_w = atomicAdd(counter, 1);
        __syncthreads();
        const int w = *s_w;
        __syncthreads();   // s_w is rewritten only after every thread has read it
        if (w >= nwork) break;
        const int4 it = work[w];
        if (!stage_tile<T, PRESS, NS, 1>(cases[it.x], it.y, it.z, it.w, base)) break;
        __syncthreads();   // the next tile's copies overwrite slots this one read
    }
}

template <typename T, int R>
size_t stage_tma_smem_bytes_r(int pressure, int n) {
    switch (n) {
        case 0: return pressure ? StageSmem<T, true, 0, R>::BYTES : StageSmem<T, false, 0, R>::BYTES;
        case 1: return pressure ? StageSmem<T, true, 1, R>::BYTES : StageSmem<T, false, 1, R>::BYTES;
        case 2: return pressure ? StageSmem<T, true, 2, R>::BYTES : StageSmem<T, false, 2, R>::BYTES;
        case 3: return pressure ? StageSmem<T, true, 3, R>::BYTES : StageSmem<T, false, 3, R>::BYTES;
        case 4: return pressure ? StageSmem<T, true, 4, R>::BYTES : StageSmem<T, false, 4, R>::BYTES;
        default: return pressure ? StageSmem<T, true, 5, R>::BYTES : StageSmem<T, false, 5, R>::BYTES;
    }
}

// dynamic shared memory of the single-case stage kernel
template <typename T>
size_t stage_tma_smem_bytes(int pressure, int n) {
    return pressure ? stage_tma_smem_bytes_r<T, stage_rows<T, true>()>(1, n)
                    : stage_tma_smem_bytes_r<T, stage_rows<T, false>()>(0, n);
}

template <typename T, bool PRESS, int NS>
static cudaError_t prep_one() {
    return cudaFuncSetAttribute(k_stage_tma<T, PRESS, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

template <typename T, bool PRESS, int NS>
static cudaError_t prep_batch() {
    return cudaFuncSetAttribute(k_stage_tma_batch<T, PRESS, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                200 * 1024);
}

template <typename T>
cudaError_t prepare_stage_tma() {
    cudaError_t e;
    if ((e = prep_one<T, false, 0>()) || (e = prep_one<T, false, 1>()) || (e = prep_one<T, false, 2>()) ||
        (e = prep_one<T, false, 3>()) || (e = prep_one<T, false, 4>()) || (e = prep_one<T, false, 5>()) ||
        (e = prep_one<T, true, 0>()) || (e = prep_one<T, true, 1>()) || (e = prep_one<T, true, 2>()) ||
        (e = prep_one<T, true, 3>()) || (e = prep_one<T, true, 4>()) || (e = prep_one<T, true, 5>()))
        return e;
    if ((e = prep_batch<T, false, 0>()) || (e = prep_batch<T, false, 1>()) || (e = prep_batch<T, false, 2>()) ||
        (e = prep_batch<T, false, 3>()) || (e = prep_batch<T, false, 4>()) || (e = prep_batch<T, false, 5>()) ||
        (e = prep_batch<T, true, 0>()) || (e = prep_batch<T, true, 1>()) || (e = prep_batch<T, true, 2>()) ||
        (e = prep_batch<T, true, 3>()) || (e = prep_batch<T, true, 4>()) || (e = prep_batch<T, true, 5>()))
        return e;
    return cudaSuccess;
}

template <typename T>
int stage_tma_batch_occupancy(int pressure) {
    int nb = 0;
    const size_t sm = stage_tma_smem_bytes_r<T, 1>(pressure, 5);
    cudaError_t e = pressure
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_stage_tma_batch<T, true, 5>, TX * TY2, sm)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_stage_tma_batch<T, false, 5>, TX * TY2, sm);
    return e == cudaSuccess && nb > 0 ? nb : 1;
}

template <typename T>
cudaError_t launch_stage_tma_batch(const StageArgsTMA<T>* cases, const int4* work, int nwork, int* counter, int n,
                                   int pressure, int nblocks, cudaStream_t s) {
    const dim3 block(TX, TY2, 1);
    const size_t sm = stage_tma_smem_bytes_r<T, 1>(pressure, n);
#define GMK_LAUNCH_B(PR)                                                                                        \
    switch (n) {                                                                                                \
        case 0: k_stage_tma_batch<T, PR, 0><<<nblocks, block, sm, s>>>(cases, work, nwork, counter); break;      \
        case 1: k_stage_tma_batch<T, PR, 1><<<nblocks, block, sm, s>>>(cases, work, nwork, counter); break;      \
        case 2: k_stage_tma_batch<T, PR, 2><<<nblocks, block, sm, s>>>(cases, work, nwork, counter); break;      \
        case 3: k_stage_tma_batch<T, PR, 3><<<nblocks, block, sm, s>>>(cases, work, nwork, counter); break;      \
        case 4: k_stage_tma_batch<T, PR, 4><<<nblocks, block, sm, s>>>(cases, work, nwork, counter); break;      \
        default: k_stage_tma_batch<T, PR, 5><<<nblocks, block, sm, s>>>(cases, work, nwork, counter); break;     \
    }
    if (pressure) {
        GMK_LAUNCH_B(true)
    } else {
        GMK_LAUNCH_B(false)
    }
#undef GMK_LAUNCH_B
    return cudaGetLastError();
}

template <typename T>
int stage_tma_occupancy(int pressure) {
    int nb = 0;
    const size_t sm = stage_tma_smem_bytes<T>(pressure, 5);
    cudaError_t e = pressure
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_stage_tma<T, true, 5>, TX * TY2, sm)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_stage_tma<T, false, 5>, TX * TY2, sm);
    return e == cudaSuccess && nb > 0 ? nb : 1;
}

template <typename T>
cudaError_t launch_stage_tma(const StageArgsTMA<T>& A, int pressure, dim3 grid, cudaStream_t s) {
    const dim3 block(TX, TY2, 1);
    const size_t sm = stage_tma_smem_bytes<T>(pressure, A.a.n);
#define GMK_LAUNCH_N(PR)                                                              \
    switch (A.a.n) {                                                                  \
        case 0: k_stage_tma<T, PR, 0><<<grid, block, sm, s>>>(A); break;              \
        case 1: k_stage_tma<T, PR, 1><<<grid, block, sm, s>>>(A); break;              \
        case 2: k_stage_tma<T, PR, 2><<<grid, block, sm, s>>>(A); break;              \
        case 3: k_stage_tma<T, PR, 3><<<grid, block, sm, s>>>(A); break;              \
        case 4: k_stage_tma<T, PR, 4><<<grid, block, sm, s>>>(A); break;              \
        default: k_stage_tma<T, PR, 5><<<grid, block, sm, s>>>(A); break;             \
    }
    if (pressure) {
        GMK_LAUNCH_N(true)
    } else {
        GMK_LAUNCH_N(false)
    }
#undef GMK_LAUNCH_N
    return cudaGetLastError();
}

#define GMK_INSTANTIATE_TMA(T)                                                                \
    template size_t stage_tma_smem_bytes<T>(int, int);                                             \
    template cudaError_t prepare_stage_tma<T>();                                              \
    template int stage_tma_occupancy<T>(int);                                                 \
    template cudaError_t launch_stage_tma<T>(const StageArgsTMA<T>&, int, dim3, cudaStream_t);                 \
    template int stage_tma_batch_occupancy<T>(int);                                                           \
    template cudaError_t launch_stage_tma_batch<T>(const StageArgsTMA<T>*, const int4*, int, int*, int, int, int, \
                                                   cudaStream_t);

}  // namespace gmk
