// gn_solve.cuh — the solve of one Gauss-Newton iteration (GetTransform's loop
// body, RGBDFusion/src/RGBDTracking.cu:184-207), run by the 32 lanes of one
// warp on inputs and outputs in the CTA's shared memory.
//
// Semantics:
//   H = H_rgb + 100 H_icp, b = b_rgb + 10 b_icp (RGBDTracking.cu:543-544);
//   error = sqrt(residualSum) / (numResidual + 6), in FP32 as the reference;
//   update = LDLT(H).solve(b): LDL^T with symmetric diagonal pivoting,
//   pseudo-inverse of D (a zero pivot -> 0), identity transpositions and no
//   factorisation if the largest diagonal is zero (or the first is NaN), L
//   columns of later zero pivots left undivided (Eigen 3's LDLT).  The pivot
//   order is fixed once from the initial |diagonal| (largest first, first on
//   ties, NaN last) where Eigen re-selects the largest remaining diagonal at
//   every step: for the positive semi-definite H of a Gauss-Newton step both
//   orders give the same solution up to rounding (1e-15 relative measured),
//   and the fixed order saves a pivot search and a row swap per step on the
//   solve's serial chain;
//   NaN in update(0): the iteration fails and the result is the identity;
//   estimate = exp(update) * estimate (SE(3) exponential);
//   the kept estimate is the one after an update whose error (measured before
//   the update) beat the level's best so far.
//
// Arithmetic: double-float.  A value is an unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi) / 2 (Dekker 1971; the TwoSum and
// TwoProduct-by-FMA transformations of Knuth and of Ogita, Rump and Oishi),
// 48 significant bits: relative error near 2^-47 per operation where FP64 has
// 2^-53.  The reference rounds H to FP32 before its FP64 factorisation
// (RGBDTracking.cu:166, 185), so the system carries 2^-24 relative error
// before the solve; the 48-bit solve adds nothing measurable to the update.
// GB300 issues one FP64 warp instruction per ~64 cycles per scheduler, so an
// FP64 solve costs its count of FP64 instructions (about 9 k cycles per
// iteration); a double-float operation is 5 to 15 FP32 instructions of 4-cycle
// latency that the scheduler issues back to back, and the solve's serial
// chain becomes a few thousand cycles.
//
// Layout: lane 0..20 holds one element (i, j), j <= i, of the lower triangle
// of H, lanes 21..26 hold b, so one elimination step updates the whole
// trailing matrix and b at once; pivot and NaN tests are integer bit
// operations on the high parts; the SE(3) exponential computes its three
// series on three lanes and one entry of [R | t] per lane.  An elimination
// step divides through the pivot's reciprocal: the approximate FP32
// reciprocal of the high part refined by one Newton-Raphson step in
// double-float, formed while the products a_ik a_jk are.
#pragma once

#include <cfloat>
#include <climits>

#include "yas_track.h"

namespace yas {

// Packed index k of the 28 products of [J | r]: rows i, columns j >= i
// (RankUpdateHessian<6,7>, TrackingUtils.h:45-58).
__device__ __forceinline__ int pack_index(int r, int c) { return 7 * r - (r * (r - 1)) / 2 + c - r; }

// ---------------------------------------------------------------- double-float
struct DF {
    float h, l;
};

__device__ __forceinline__ DF df(float h) { return DF{h, 0.0f}; }
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }

// a + b for |a| >= |b| (or a == 0): FastTwoSum, s = fl(a + b) exactly split.
__device__ __forceinline__ DF df_fast(float a, float b) {
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// a + b for any a, b: TwoSum, s = fl(a + b), s + e = a + b exactly.
__device__ __forceinline__ DF df_two(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ DF df_add(DF a, DF b) {
    const DF s = df_two(a.h, b.h);
    return df_fast(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return df_fast(p, e);
}

// a * b + c
__device__ __forceinline__ DF df_fma(DF a, DF b, DF c) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    const DF s = df_two(p, c.h);
    return df_fast(s.h, __fadd_rn(s.l, __fadd_rn(e, c.l)));
}

__device__ __forceinline__ double df_to_double(DF a) { return (double)a.h + (double)a.l; }

// Nearest double-float of x (hi = x rounded to FP32, lo = the rest rounded).
__device__ __forceinline__ DF df_from_double(double x) {
    const float h = (float)x;
    return DF{h, (float)(x - (double)h)};
}

// The range in which the FP32 reciprocal of the high part is a normal number
// with room for the refinement: 1e-30 < |x.h| < 1e30.
__device__ __forceinline__ bool df_seed_range(DF x) {
    const unsigned a = __float_as_uint(x.h) & 0x7fffffffu;
    return a > 0x0da24260u && a < 0x7149f2cau;
}

// 1 / d: r0 = the hardware's approximate FP32 reciprocal of d.h (relative
// error below 2^-22), e = 1 - d r0 (1 - fl(d.h r0) is exact: Sterbenz),
// r = r0 + r0 e, one Newton-Raphson step: relative error below 2^-43.  A
// pivot outside the seed range is first scaled by 2^64 or 2^-64 (exact) and
// the reciprocal scaled back, without a branch (pivots of a Gauss-Newton
// system stay far inside: its entries are sums of squared image and depth
// gradients).
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ DF df_rcp(DF d) {
    const unsigned ab = __float_as_uint(d.h) & 0x7fffffffu;
    const float sc = ab <= 0x0da24260u ? 0x1p64f : (ab >= 0x7149f2cau ? 0x1p-64f : 1.0f);
    const float dh = __fmul_rn(d.h, sc), dl = __fmul_rn(d.l, sc);
    const float r0 = rcp_approx(dh);
    const float p = __fmul_rn(dh, r0);
    const float pe = __fmaf_rn(dh, r0, -p);
    const float e = __fmaf_rn(-dl, r0, __fsub_rn(__fsub_rn(1.0f, p), pe));
    const DF r = df_fast(r0, __fmul_rn(r0, e));
    return DF{__fmul_rn(r.h, sc), __fmul_rn(r.l, sc)};
}

// a / x: a times the refined reciprocal in the seed range, an FP64 division
// outside it (there 1 / x itself could leave the normal FP32 range of a low
// part); yas_check_div_seeded evaluates it for the tests.
__device__ __forceinline__ DF df_div(DF a, DF x) {
    if (!df_seed_range(x)) return df_from_double(df_to_double(a) / df_to_double(x));
    return df_mul(a, df_rcp(x));
}

__device__ __forceinline__ DF df_shfl(DF a, int src) {
    return DF{__shfl_sync(0xffffffffu, a.h, src), __shfl_sync(0xffffffffu, a.l, src)};
}

__device__ __forceinline__ DF df_sel3(int i, DF x, DF y, DF z) { return i == 0 ? x : (i == 1 ? y : z); }

// ---------------------------------------------------------------- solve state
// Inputs, state and outputs of the solve, in the shared memory of the CTA
// that runs it; every FP64 quantity of the reference is a double-float pair.
struct SolveShared {
    // pass A totals: 0..26 ICP H|b, 27 ICP sum r^2, 28 ICP count, 29..31 RGB moments
    float Ah[32], Al[32];
    // pass B totals: 0..26 RGB H|b, 27 RGB sum w r^2
    float Bh[32], Bl[32];
    // estimate state (in: before the iteration; out: after it)
    float esth[12], estl[12];
    float besth[12], bestl[12];
    float last_error;
    int n_success, n_iter, failed, level_of_last;
    float Tf[12];  // the estimate rounded to FP32 (= esth)
    float huber_th;
    // outputs of the last solve
    float Hh[36], Hl[36], bh[6], bl[6], uh[6], ul[6];
    float stats[3];  // residualSum, numResidual, huber_th (FP32 in the reference)
    float xsh[8], xsl[8];  // solution scatter (undoing the pivot permutation)
    int perm[8];           // static pivot order: perm[p] = the row pivoted at step p
};
__shared__ SolveShared g_solve;

// Sets total i of pass A (which = 0) or B (which = 1) from a compensated FP32
// pair (h, l): normalised so the high part is the total rounded to FP32.
__device__ __forceinline__ void set_total(int which, int i, float h, float l) {
    const DF v = df_two(h, l);
    if (which == 0) {
        g_solve.Ah[i] = v.h;
        g_solve.Al[i] = v.l;
    } else {
        g_solve.Bh[i] = v.h;
        g_solve.Bl[i] = v.l;
    }
}

__device__ __forceinline__ void set_total_double(int which, int i, double x) {
    const DF v = df_from_double(x);
    set_total(which, i, v.h, v.l);
}

__device__ __forceinline__ DF total(int which, int i) {
    return which == 0 ? DF{g_solve.Ah[i], g_solve.Al[i]} : DF{g_solve.Bh[i], g_solve.Bl[i]};
}

__device__ __forceinline__ DF combine_sys(int mode, DF a, DF b, float wa) {
    return mode == YAS_TRACK_RGBD ? df_fma(df(wa), a, b) : (mode == YAS_TRACK_RGB ? b : a);
}

__device__ __forceinline__ int tri_lane(int i, int j) { return i * (i + 1) / 2 + j; }  // i >= j

__device__ __forceinline__ float sel3f(int i, float x, float y, float z) { return i == 0 ? x : (i == 1 ? y : z); }

constexpr unsigned kAbsMaskF = 0x7fffffffu;
constexpr unsigned kInfBitsF = 0x7f800000u;

// The solve (warp 0; every lane must call it).  Reads g_solve's totals and
// estimate state, writes the new state and the outputs back to g_solve.
// Inlined into kernels with registers to spare (gn_solve_inline), called
// (gn_solve) from the 64-register ones, where inlining adds spills.
__device__ __forceinline__ void gn_solve_inline(int mode, int no_update, int first_of_level, int level) {
    SolveShared &S = g_solve;
    constexpr unsigned kAll = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31);
    // ---- this lane's element: (ei, ej) of the lower triangle, or b[ei] (ej = 6)
    int ei = 0, ej = 7;
    if (lane < 21) {
        ei = (lane >= 1) + (lane >= 3) + (lane >= 6) + (lane >= 10) + (lane >= 15);
        ej = lane - tri_lane(ei, 0);
    } else if (lane < 27) {
        ei = lane - 21;
        ej = 6;
    }
    const bool isb = ej == 6, ism = ej < 6;
    DF a = df(0.0f);
    if (ej <= 6) {
        const int k = pack_index(min(ei, ej), max(ei, ej));
        a = combine_sys(mode, total(0, k), total(1, k), isb ? 10.0f : 100.0f);
    }
    if (ism) {
        S.Hh[ei * 6 + ej] = a.h;
        S.Hl[ei * 6 + ej] = a.l;
        S.Hh[ej * 6 + ei] = a.h;
        S.Hl[ej * 6 + ei] = a.l;
    } else if (isb) {
        S.bh[ei] = a.h;
        S.bl[ei] = a.l;
    }
    // residualSum and numResidual are FP32 in the reference: the high parts
    // (each total is normalised, so its high part is the total rounded to FP32)
    const float residualSum = mode == YAS_TRACK_RGB ? S.Bh[27] : S.Ah[27];
    const float numResidual = mode == YAS_TRACK_ICP ? S.Ah[28] : S.Ah[29];
    if (lane == 0) {
        S.stats[0] = residualSum;
        S.stats[1] = numResidual;
        S.stats[2] = S.huber_th;
    }
    if (no_update) {
        __syncwarp();
        return;
    }
    // acceptance on the error measured before the update, decided by every
    // lane now so that its division and square root overlap the factorisation
    const float error = sqrtf(residualSum) / (numResidual + 6.0f);
    const float last = first_of_level ? FLT_MAX : S.last_error;
    const bool accept = error < last;
    // ---- LDL^T on [H | b] with a static pivot order: the diagonal's initial
    // |values|, largest first (first on ties), applied as one symmetric
    // permutation; the factorisation itself divides through the refined
    // reciprocal of each pivot
    int orig = ei;  // b lanes: original index of the row they hold
    bool broke = false;
    {
        const unsigned ab0 = __float_as_uint(a.h) & kAbsMaskF;
        const int key0 = (ism && ei == ej) ? (ab0 > kInfBitsF ? -1 : (int)ab0) : -2;
        // lane 5q + r' (r' < 5) asks whether row r (the r'-th row other than
        // q) ranks before row q; the rank of q counts its five answers
        const int pq = lane / 5, pr0 = lane - 5 * pq, pr = pr0 < pq ? pr0 : pr0 + 1;
        const int kq = __shfl_sync(kAll, key0, lane < 30 ? tri_lane(pq, pq) : 0);
        const int kr = __shfl_sync(kAll, key0, lane < 30 ? tri_lane(pr, pr) : 0);
        const unsigned before = __ballot_sync(kAll, lane < 30 && (kr > kq || (kr == kq && pr < pq)));
        // perm[p] = the row of rank p
        if (lane < 6) S.perm[__popc((before >> (5 * lane)) & 0x1fu)] = lane;
        const int kmax = __reduce_max_sync(kAll, key0 == -2 ? INT_MIN : key0);
        const int k0 = __shfl_sync(kAll, key0, 0);
        __syncwarp();
        // no factorisation when the largest diagonal is zero or the first is NaN
        broke = kmax <= 0 || k0 == -1;
        if (!broke) {
            const int pi = ism || isb ? S.perm[ei] : 0;
            const int pj = ism ? S.perm[ej] : 0;
            const int src = ism ? (pi >= pj ? tri_lane(pi, pj) : tri_lane(pj, pi)) : (isb ? 21 + pi : lane);
            a = df_shfl(a, src);
            if (isb) orig = pi;
        }
    }
    DF rk = df(0.0f);  // b lane i: reciprocal of pivot i (for D^+ y)
    if (!broke) {
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const bool upd = ei > k && ((ism && ej > k) || isb);
            const int src_l = upd ? tri_lane(ei, k) : lane;
            const int src_x = upd ? (isb ? 21 + k : tri_lane(ej, k)) : lane;
            const DF d = df_shfl(a, tri_lane(k, k));
            const DF lik = df_shfl(a, src_l);
            const DF ajk = df_shfl(a, src_x);
            const unsigned db = __float_as_uint(d.h) & kAbsMaskF;
            const bool valid = db != 0u && db <= kInfBitsF;
            const DF t = df_mul(lik, ajk);
            DF r = df(1.0f);  // undivided for a zero pivot
            if (valid) r = db == kInfBitsF ? df(0.0f) : df_rcp(d);
            const DF na = df_fma(df_neg(t), r, a);
            const bool colk = ism && ej == k && ei > k;
            const DF nl = df_mul(a, r);
            if (upd && (isb || valid)) a = na;
            if (colk) a = nl;
            if (isb && ei == k) rk = r;
        }
    }
    if (broke) {  // forward substitution with the unfactored lower triangle
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const DF yj = df_shfl(a, 21 + j);
            const bool u = isb && ei > j;
            const DF lij = df_shfl(a, u ? tri_lane(ei, j) : lane);
            const DF na = df_fma(df_neg(lij), yj, a);
            if (u) a = na;
        }
    }
    {  // D^+ y on the b lanes (a zero or NaN pivot gives 0; an infinite one 0):
       // times the pivot's reciprocal from the factorisation (the diagonal is
       // final once its step has run), a division when nothing was factorised
        const DF dd = df_shfl(a, isb ? tri_lane(ei, ei) : lane);
        const unsigned db = __float_as_uint(dd.h) & kAbsMaskF;
        if (isb) a = (db != 0u && db < kInfBitsF) ? (broke ? df_div(a, dd) : df_mul(a, rk)) : df(0.0f);
    }
    // ---- L^T z = y: b_i -= L(j, i) z_j for j > i
#pragma unroll
    for (int j = 5; j > 0; --j) {
        const DF zj = df_shfl(a, 21 + j);
        const bool u = isb && ei < j;
        const DF lji = df_shfl(a, u ? tri_lane(j, ei) : lane);
        const DF na = df_fma(df_neg(lji), zj, a);
        if (u) a = na;
    }
    // ---- x = P^T z
    if (isb) {
        S.xsh[orig] = a.h;
        S.xsl[orig] = a.l;
    }
    __syncwarp();
    DF u[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) u[q] = DF{S.xsh[q], S.xsl[q]};
    if (lane < 6) {
        S.uh[lane] = S.xsh[lane];
        S.ul[lane] = S.xsl[lane];
    }
    if ((__float_as_uint(u[0].h) & kAbsMaskF) > kInfBitsF) {
        if (lane == 0) S.failed = kFailNumeric;
        if (lane < 12) {
            S.besth[lane] = (lane % 5 == 0) ? 1.0f : 0.0f;
            S.bestl[lane] = 0.0f;
        }
        __syncwarp();
        return;
    }
    // ---- SE(3) exponential: R = I + cA W + cB W^2, t = v + cB (w x v) + cC W^2 v,
    // W = hat(w), W^2 = w w^T - th^2 I; lane i*4 + q computes E(i, q) (q < 3)
    // or t_i (q = 3) with one instruction sequence:
    //   E(i, q) = d_iq + cA W_iq + cB (w_i w_q - d_iq th^2)
    //   t_i     = v_i  + cB (w x v)_i + cC (w_i (w . v) - th^2 v_i)
    const DF wx = u[3], wy = u[4], wz = u[5];
    const DF th2 = df_fma(wx, wx, df_fma(wy, wy, df_mul(wz, wz)));
    DF cA, cB, cC;
    if (th2.h < 1e-2f) {
        // Taylor series in th^2 to the th^8 term (truncation below 3e-18) of
        // sin(th)/th, (1-cos th)/th^2 and (th-sin th)/th^3; lane r % 3
        // evaluates series r % 3: the terms of order th^4 and higher in FP32
        // (they are below th^4 / 120 <= 1e-6 of the sum), the first two in
        // double-float (coefficients split into high and low parts)
        const int sr = lane % 3;
        const float p4 = sel3f(sr, (float)(1.0 / 362880.0), (float)(1.0 / 3628800.0), (float)(1.0 / 39916800.0));
        const float p3 = sel3f(sr, (float)(-1.0 / 5040.0), (float)(-1.0 / 40320.0), (float)(-1.0 / 362880.0));
        const float p2 = sel3f(sr, (float)(1.0 / 120.0), (float)(1.0 / 720.0), (float)(1.0 / 5040.0));
        constexpr float k6h = (float)(1.0 / 6.0), k24h = (float)(1.0 / 24.0), k120h = (float)(1.0 / 120.0);
        const DF p1 = DF{sel3f(sr, -k6h, -k24h, -k120h),
                         sel3f(sr, (float)(-1.0 / 6.0 + (double)k6h), (float)(-1.0 / 24.0 + (double)k24h),
                               (float)(-1.0 / 120.0 + (double)k120h))};
        const DF p0 = DF{sel3f(sr, 1.0f, 0.5f, k6h), sel3f(sr, 0.0f, 0.0f, (float)(1.0 / 6.0 - (double)k6h))};
        const float q = __fmaf_rn(th2.h, __fmaf_rn(th2.h, p4, p3), p2);
        const DF pc = df_fma(th2, df_fma(th2, df(q), p1), p0);
        cA = df_shfl(pc, 0);
        cB = df_shfl(pc, 1);
        cC = df_shfl(pc, 2);
    } else {
        // rotations above 0.1 rad per iteration: FP64 (rare)
        const double t2 = df_to_double(th2);
        const double th = sqrt(t2);
        double sn, cs;
        sincos(th, &sn, &cs);
        cA = df_from_double(sn / th);
        cB = df_from_double((1.0 - cs) / t2);
        cC = df_from_double((th - sn) / (t2 * th));
    }
    const int i = lane < 12 ? lane >> 2 : 0, q = lane & 3;
    const bool tl = q == 3;
    const DF wi = df_sel3(i, wx, wy, wz), ui = df_sel3(i, u[0], u[1], u[2]);
    const DF wq = df_sel3(q, wx, wy, wz);
    // (w x v)_i = w_{i+1} v_{i+2} - w_{i+2} v_{i+1} (indices mod 3)
    const int i1 = i == 2 ? 0 : i + 1, i2 = i == 0 ? 2 : i - 1;
    const DF wxv = df_fma(df_sel3(i1, wx, wy, wz), df_sel3(i2, u[0], u[1], u[2]),
                          df_neg(df_mul(df_sel3(i2, wx, wy, wz), df_sel3(i1, u[0], u[1], u[2]))));
    const DF wdv = df_fma(wx, u[0], df_fma(wy, u[1], df_mul(wz, u[2])));
    // W_iq = -eps_iqm w_m
    DF Wiq = df(0.0f);
    if (i != q && !tl) {
        const int m = 3 - i - q;
        const DF wm = df_sel3(m, wx, wy, wz);
        Wiq = (q == (i + 1) % 3) ? df_neg(wm) : wm;
    }
    const bool diag = i == q;
    const DF thu = df_mul(th2, ui);
    const DF c1 = tl ? cB : cA, y1 = tl ? wxv : Wiq, x0 = tl ? ui : df(diag ? 1.0f : 0.0f);
    const DF c2 = tl ? cC : cB, y2 = tl ? wdv : wq, z2 = tl ? df_neg(thu) : (diag ? df_neg(th2) : df(0.0f));
    const DF ent = df_fma(c2, df_fma(wi, y2, z2), df_fma(c1, y1, x0));
    // ---- estimate = E * estimate, entry (i, q) on lane i*4 + q
    const DF E0 = df_shfl(ent, i * 4 + 0), E1 = df_shfl(ent, i * 4 + 1);
    const DF E2 = df_shfl(ent, i * 4 + 2), ti = df_shfl(ent, i * 4 + 3);
    const DF o = df_fma(E0, DF{S.esth[q], S.estl[q]},
                        df_fma(E1, DF{S.esth[4 + q], S.estl[4 + q]},
                               df_fma(E2, DF{S.esth[8 + q], S.estl[8 + q]}, tl ? ti : df(0.0f))));
    // ---- the new state
    if (lane == 0) {
        S.last_error = accept ? error : last;
        S.n_success += accept ? 1 : 0;
        S.n_iter += 1;
        S.level_of_last = level;
    }
    if (lane < 12) {
        S.esth[lane] = o.h;
        S.estl[lane] = o.l;
        S.Tf[lane] = o.h;
        if (accept) {
            S.besth[lane] = o.h;
            S.bestl[lane] = o.l;
        }
    }
    __syncwarp();
}

__device__ __noinline__ void gn_solve(int mode, int no_update, int first_of_level, int level) {
    gn_solve_inline(mode, no_update, first_of_level, level);
}

// Threads 0..31 load the estimate state of `st` into g_solve (the caller sets
// g_solve.huber_th and the pass totals).
__device__ __forceinline__ void load_solve_state(const GNState *st) {
    const int t = (int)threadIdx.x;
    if (t < 12) {
        const DF e = df_from_double(__ldcg(&st->est[t]));
        const DF b = df_from_double(__ldcg(&st->best[t]));
        g_solve.esth[t] = e.h;
        g_solve.estl[t] = e.l;
        g_solve.besth[t] = b.h;
        g_solve.bestl[t] = b.l;
        g_solve.Tf[t] = __ldcg(&st->Tf[t]);
    } else if (t == 12) {
        g_solve.last_error = (float)__ldcg(&st->last_error);
    } else if (t == 13) {
        g_solve.n_success = __ldcg(&st->n_success);
        g_solve.n_iter = __ldcg(&st->n_iter);
        g_solve.failed = __ldcg(&st->failed);
        g_solve.level_of_last = __ldcg(&st->level_of_last);
    }
}

// Threads 0..31 write g_solve's state and last outputs to `st` (double-float
// pairs widened to FP64, exactly).
__device__ __forceinline__ void publish_solve(GNState *st) {
    const int t = (int)threadIdx.x;
    if (t >= 32) return;
    if (t < 12) {
        st->est[t] = df_to_double(DF{g_solve.esth[t], g_solve.estl[t]});
        st->best[t] = df_to_double(DF{g_solve.besth[t], g_solve.bestl[t]});
        st->Tf[t] = g_solve.Tf[t];
    }
    for (int k = t; k < 36; k += 32) st->H[k] = df_to_double(DF{g_solve.Hh[k], g_solve.Hl[k]});
    if (t < 6) {
        st->b[t] = df_to_double(DF{g_solve.bh[t], g_solve.bl[t]});
        st->last_update[t] = df_to_double(DF{g_solve.uh[t], g_solve.ul[t]});
    }
    if (t < 3) st->stats[t] = (double)g_solve.stats[t];
    if (t == 3) st->stats[3] = df_to_double(DF{g_solve.Ah[28], g_solve.Al[28]});
    if (t == 0) {
        st->last_error = (double)g_solve.last_error;
        st->n_success = g_solve.n_success;
        st->n_iter = g_solve.n_iter;
        st->failed = g_solve.failed;
        st->level_of_last = g_solve.level_of_last;
        st->huber_th = g_solve.huber_th;
    }
}

}  // namespace yas
