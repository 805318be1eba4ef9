// gn_solve.cuh — the FP64 solve of one Gauss-Newton iteration (GetTransform's
// loop body, RGBDFusion/src/RGBDTracking.cu:184-207), run by the 32 lanes of
// one warp on inputs and outputs in the CTA's shared memory.
//
// Semantics:
//   H = H_rgb + 100 H_icp, b = b_rgb + 10 b_icp (RGBDTracking.cu:543-544);
//   error = sqrt(residualSum) / (numResidual + 6), in FP32 as the reference;
//   update = LDLT(H).solve(b) in FP64: LDL^T with symmetric diagonal
//   pivoting, pseudo-inverse of D (|d| <= 1/DBL_MAX -> 0), identity
//   transpositions and no factorisation if the largest diagonal is zero (or
//   the first is NaN), L columns of later zero pivots left undivided (Eigen 3's
//   LDLT).  The pivot order is fixed once from the initial |diagonal| (largest
//   first, first on ties, NaN last) where Eigen re-selects the largest
//   remaining diagonal at every step: for the positive semi-definite H of a
//   Gauss-Newton step both orders give the same solution up to rounding
//   (1e-15 relative measured), and the fixed order saves a pivot search and a
//   row swap per step on the solve's serial chain;
//   NaN in update(0): the iteration fails and the result is the identity;
//   estimate = exp(update) * estimate (SE(3) exponential, FP64);
//   the kept estimate is the one after an update whose error (measured before
//   the update) beat the level's best so far.
//
// GB300 executes one FP64 warp instruction per ~64 cycles per scheduler, with
// or without dependencies, so the cost of the solve is its count of FP64 warp
// instructions.  The layout minimises that count: lane 0..20 holds one element
// (i, j), j <= i, of the lower triangle of H, lanes 21..26 hold b, so one
// elimination step is five FP64 instructions for the whole trailing matrix
// and b; pivot tests, NaN tests and reciprocal seeds are integer bit
// operations; the SE(3) exponential computes its three series on three lanes
// and one entry of [R | t] per lane.  An elimination step divides through the
// pivot's reciprocal (an FP32 seed refined by one Newton-Raphson step), so the
// products a_ik a_jk of the trailing update are formed while the reciprocal is
// refined.
#pragma once

#include <cfloat>

#include "yas_track.h"

namespace yas {

// Packed index k of the 28 products of [J | r]: rows i, columns j >= i
// (RankUpdateHessian<6,7>, TrackingUtils.h:45-58).
__device__ __forceinline__ int pack_index(int r, int c) { return 7 * r - (r * (r - 1)) / 2 + c - r; }

// Inputs, state and outputs of the solve, in the shared memory of the CTA
// that runs it.
struct SolveShared {
    double A[32];  // pass A totals: 0..26 ICP H|b, 27 ICP sum r^2, 28 ICP count, 29..31 RGB moments
    double B[32];  // pass B totals: 0..26 RGB H|b, 27 RGB sum w r^2
    // estimate state (in: before the iteration; out: after it)
    double est[12];
    double best[12];
    double last_error;
    int n_success, n_iter, failed, level_of_last;
    float Tf[12];
    float huber_th;
    // outputs of the last solve
    double H[36], b[6], stats[4], last_update[6];
    double xs[8];  // solution scatter (undoing the pivot permutation)
};
__shared__ SolveShared g_solve;

constexpr unsigned long long kAbsMask = 0x7fffffffffffffffull;
constexpr unsigned long long kInfBits = 0x7ff0000000000000ull;

__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & kAbsMask;
}
// 1e-30 < |x| < 1e30 (the range of the FP32 reciprocal seed)
__device__ __forceinline__ bool seed_range(double x) {
    const unsigned long long a = abs_bits(x);
    return a > 0x39b4484bfeebc2a0ull && a < 0x46293e5939a08ceaull;
}

// FP64 value of the FP32 reciprocal of x (x truncated to FP32), for
// 1e-30 < |x| < 1e30, by bit manipulation and one FP32 reciprocal.
__device__ __forceinline__ double rcp_seed(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned e = (hi >> 20) & 0x7ffu;
    const unsigned fb = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rb = __float_as_uint(__frcp_rn(__uint_as_float(fb)));
    const unsigned ef = (rb >> 23) & 0xffu;
    const unsigned hi2 = (rb & 0x80000000u) | ((ef + 896u) << 20) | ((rb & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi2, (int)((rb & 0x7fffffu) << 29));
}

// a / x by one Newton-Raphson refinement of an FP32 reciprocal seed: with the
// seed r = (1 - d) / x (|d| < 2^-22), e = 1 - x r = d and a r (1 + e) =
// (a / x)(1 - d^2), a relative error below 2^-44 plus the FP64 roundings
// (far below the ~1e-7 precision of the FP32-accumulated system it is applied
// to); outside the seed range an IEEE division.  yas_check_div_seeded
// evaluates it for the tests.
__device__ __forceinline__ double div_seeded(double a, double x) {
    if (!seed_range(x)) return a / x;
    const double r = rcp_seed(x);
    const double q0 = a * r;
    return fma(q0, fma(-x, r, 1.0), q0);
}

// (float)x, rounded to nearest even, by integer operations for a value in the
// normal FP32 range (the conversion instruction otherwise; same result).
__device__ __forceinline__ float to_float_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    if (e < 897u || e > 1150u) return (float)x;
    const unsigned long long m = b & 0xfffffffffffffull;
    unsigned f = (unsigned)(b >> 63) << 31 | (e - 896u) << 23 | (unsigned)(m >> 29);
    const unsigned rem = (unsigned)(m & 0x1fffffffull);
    if (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ++f;  // a carry rounds into the exponent
    return __uint_as_float(f);
}

__device__ __forceinline__ double combine_sys(int mode, double a, double b, double wa) {
    return mode == YAS_TRACK_RGBD ? fma(wa, a, b) : (mode == YAS_TRACK_RGB ? b : a);
}

__device__ __forceinline__ int tri_lane(int i, int j) { return i * (i + 1) / 2 + j; }  // i >= j

__device__ __forceinline__ double sel3(int i, double x, double y, double z) { return i == 0 ? x : (i == 1 ? y : z); }

// The solve (warp 0; every lane must call it).  Reads g_solve.A/B and the
// estimate state, writes the new state and the outputs back to g_solve.
__device__ __noinline__ void gn_solve(int mode, int no_update, int first_of_level, int level) {
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
    double a = 0.0;
    if (ej <= 6) a = combine_sys(mode, S.A[pack_index(min(ei, ej), max(ei, ej))], S.B[pack_index(min(ei, ej), max(ei, ej))],
                                 isb ? 10.0 : 100.0);
    if (ism) {
        S.H[ei * 6 + ej] = a;
        S.H[ej * 6 + ei] = a;
    } else if (isb) {
        S.b[ei] = a;
    }
    // residualSum and numResidual are FP32 in the reference
    const float residualSum = to_float_rn(mode == YAS_TRACK_RGB ? S.B[27] : S.A[27]);
    const float numResidual = to_float_rn(mode == YAS_TRACK_ICP ? S.A[28] : S.A[29]);
    if (lane == 0) {
        S.stats[0] = (double)residualSum;
        S.stats[1] = (double)numResidual;
        S.stats[2] = (double)S.huber_th;
        S.stats[3] = S.A[28];
    }
    if (no_update) {
        __syncwarp();
        return;
    }
    // ---- LDL^T on [H | b] with a static pivot order: the diagonal's initial
    // |values|, largest first (first on ties), applied as one symmetric
    // permutation; the factorisation itself divides through the refined
    // reciprocal of each pivot
    int orig = ei;  // b lanes: original index of the row they hold
    bool broke = false;
    {
        const unsigned long long ab0 = abs_bits(a);
        const long long key0 = (ism && ei == ej) ? (ab0 > kInfBits ? -1LL : (long long)ab0) : -2LL;
        long long kd[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) kd[q] = __shfl_sync(kAll, key0, tri_lane(q, q));
        int pos[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            int rq = 0;
#pragma unroll
            for (int r = 0; r < 6; ++r) rq += (kd[r] > kd[q] || (kd[r] == kd[q] && r < q)) ? 1 : 0;
            pos[q] = rq;
        }
        int inv[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) inv[pos[q]] = q;
        // no factorisation when the largest diagonal is zero or the first is NaN
        const long long kmax = kd[inv[0]];
        broke = kmax <= 0 || kd[0] == -1LL;
        if (!broke) {
            const int pi = ism || isb ? inv[ei] : 0;
            const int pj = ism ? inv[ej] : 0;
            const int src = ism ? (pi >= pj ? tri_lane(pi, pj) : tri_lane(pj, pi)) : (isb ? 21 + pi : lane);
            a = __shfl_sync(kAll, a, src);
            if (isb) orig = pi;
        }
    }
    if (!broke) {
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const bool upd = ei > k && ((ism && ej > k) || isb);
            const int src_l = upd ? tri_lane(ei, k) : lane;
            const int src_x = upd ? (isb ? 21 + k : tri_lane(ej, k)) : lane;
            const double d = __shfl_sync(kAll, a, tri_lane(k, k));
            const double lik = __shfl_sync(kAll, a, src_l);
            const double ajk = __shfl_sync(kAll, a, src_x);
            const unsigned long long db = abs_bits(d);
            const bool valid = db != 0ull && db <= kInfBits;
            const double t = lik * ajk;
            double r = 1.0;  // undivided for a zero pivot
            if (valid) {
                if (seed_range(d)) {
                    const double r0 = rcp_seed(d);
                    r = fma(r0, fma(-d, r0, 1.0), r0);
                } else {
                    r = 1.0 / d;
                }
            }
            const double na = fma(-t, r, a);
            const bool colk = ism && ej == k && ei > k;
            const double nl = a * r;
            if (upd && (isb || valid)) a = na;
            if (colk) a = nl;
        }
    }
    if (broke) {  // forward substitution with the unfactored lower triangle
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const double yj = __shfl_sync(kAll, a, 21 + j);
            const bool u = isb && ei > j;
            const double lij = __shfl_sync(kAll, a, u ? tri_lane(ei, j) : lane);
            const double na = fma(-lij, yj, a);
            if (u) a = na;
        }
    }
    {  // D^+ y on the b lanes
        const double dd = __shfl_sync(kAll, a, isb ? tri_lane(ei, ei) : lane);
        const unsigned long long db = abs_bits(dd);
        if (isb) a = (db > 0x0004000000000000ull && db <= kInfBits) ? div_seeded(a, dd) : 0.0;
    }
    // ---- L^T z = y: b_i -= L(j, i) z_j for j > i
#pragma unroll
    for (int j = 5; j > 0; --j) {
        const double zj = __shfl_sync(kAll, a, 21 + j);
        const bool u = isb && ei < j;
        const double lji = __shfl_sync(kAll, a, u ? tri_lane(j, ei) : lane);
        const double na = fma(-lji, zj, a);
        if (u) a = na;
    }
    // ---- x = P^T z
    if (isb) S.xs[orig] = a;
    __syncwarp();
    double u[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) u[q] = S.xs[q];
    if (lane < 6) S.last_update[lane] = S.xs[lane];
    if (abs_bits(u[0]) > kInfBits) {
        if (lane == 0) S.failed = kFailNumeric;
        if (lane < 12) S.best[lane] = (lane % 5 == 0) ? 1.0 : 0.0;
        __syncwarp();
        return;
    }
    // ---- SE(3) exponential: R = I + cA W + cB W^2, t = v + cB (w x v) + cC W^2 v,
    // W = hat(w), W^2 = w w^T - th^2 I; lane i*4 + q computes E(i, q) (q < 3)
    // or t_i (q = 3) with one instruction sequence:
    //   E(i, q) = d_iq + cA W_iq + cB (w_i w_q - d_iq th^2)
    //   t_i     = v_i  + cB (w x v)_i + cC (w_i (w . v) - th^2 v_i)
    const double wx = u[3], wy = u[4], wz = u[5];
    const double th2 = fma(wx, wx, fma(wy, wy, wz * wz));
    double cA, cB, cC;
    if (abs_bits(th2) < 0x3f847ae147ae147bull) {  // th^2 < 1e-2
        // Taylor series in th^2 to the th^8 term (truncation below 3e-18) of
        // sin(th)/th, (1-cos th)/th^2 and (th-sin th)/th^3; lane r % 3
        // evaluates series r % 3 (coefficients selected from immediates)
        const int sr = lane % 3;
        const double p4 = sel3(sr, 1.0 / 362880.0, 1.0 / 3628800.0, 1.0 / 39916800.0);
        const double p3 = sel3(sr, -1.0 / 5040.0, -1.0 / 40320.0, -1.0 / 362880.0);
        const double p2 = sel3(sr, 1.0 / 120.0, 1.0 / 720.0, 1.0 / 5040.0);
        const double p1 = sel3(sr, -1.0 / 6.0, -1.0 / 24.0, -1.0 / 120.0);
        const double p0 = sel3(sr, 1.0, 0.5, 1.0 / 6.0);
        const double pc = fma(th2, fma(th2, fma(th2, fma(th2, p4, p3), p2), p1), p0);
        cA = __shfl_sync(kAll, pc, 0);
        cB = __shfl_sync(kAll, pc, 1);
        cC = __shfl_sync(kAll, pc, 2);
    } else {
        const double th = sqrt(th2);
        double sn, cs;
        sincos(th, &sn, &cs);
        cA = sn / th;
        cB = (1.0 - cs) / th2;
        cC = (th - sn) / (th2 * th);
    }
    const int i = lane < 12 ? lane >> 2 : 0, q = lane & 3;
    const bool tl = q == 3;
    const double wi = sel3(i, wx, wy, wz), ui = sel3(i, u[0], u[1], u[2]);
    const double wq = sel3(q, wx, wy, wz);
    // (w x v)_i = w_{i+1} v_{i+2} - w_{i+2} v_{i+1} (indices mod 3)
    const int i1 = i == 2 ? 0 : i + 1, i2 = i == 0 ? 2 : i - 1;
    const double wxv = fma(sel3(i1, wx, wy, wz), sel3(i2, u[0], u[1], u[2]), -(sel3(i2, wx, wy, wz) * sel3(i1, u[0], u[1], u[2])));
    const double wdv = fma(wx, u[0], fma(wy, u[1], wz * u[2]));
    // W_iq = -eps_iqm w_m
    double Wiq = 0.0;
    if (i != q && !tl) {
        const int m = 3 - i - q;
        const double wm = sel3(m, wx, wy, wz);
        Wiq = (q == (i + 1) % 3) ? -wm : wm;
    }
    const bool diag = i == q;
    const double thu = th2 * ui;
    const double c1 = tl ? cB : cA, y1 = tl ? wxv : Wiq, x0 = tl ? ui : (diag ? 1.0 : 0.0);
    const double c2 = tl ? cC : cB, y2 = tl ? wdv : wq, z2 = tl ? -thu : (diag ? -th2 : 0.0);
    const double ent = fma(c2, fma(wi, y2, z2), fma(c1, y1, x0));
    // ---- estimate = E * estimate, entry (i, q) on lane i*4 + q
    const double E0 = __shfl_sync(kAll, ent, i * 4 + 0), E1 = __shfl_sync(kAll, ent, i * 4 + 1);
    const double E2 = __shfl_sync(kAll, ent, i * 4 + 2), ti = __shfl_sync(kAll, ent, i * 4 + 3);
    const double o = fma(E0, S.est[q], fma(E1, S.est[4 + q], fma(E2, S.est[8 + q], tl ? ti : 0.0)));
    // ---- acceptance on the error measured before the update
    const float error = sqrtf(residualSum) / (numResidual + 6.0f);
    int accept = 0;
    if (lane == 0) {
        const double last = first_of_level ? (double)FLT_MAX : S.last_error;
        accept = (double)error < last;
        S.last_error = accept ? (double)error : last;
        S.n_success += accept ? 1 : 0;
        S.n_iter += 1;
        S.level_of_last = level;
    }
    accept = __shfl_sync(kAll, accept, 0);
    __syncwarp();
    if (lane < 12) {
        S.est[lane] = o;
        S.Tf[lane] = (float)o;
        if (accept) S.best[lane] = o;
    }
    __syncwarp();
}

// Threads 0..31 load the estimate state of `st` into g_solve (the caller sets
// g_solve.huber_th and the pass totals).
__device__ __forceinline__ void load_solve_state(const GNState *st) {
    const int t = (int)threadIdx.x;
    if (t < 12) {
        g_solve.est[t] = __ldcg(&st->est[t]);
        g_solve.best[t] = __ldcg(&st->best[t]);
        g_solve.Tf[t] = __ldcg(&st->Tf[t]);
    } else if (t == 12) {
        g_solve.last_error = __ldcg(&st->last_error);
    } else if (t == 13) {
        g_solve.n_success = __ldcg(&st->n_success);
        g_solve.n_iter = __ldcg(&st->n_iter);
        g_solve.failed = __ldcg(&st->failed);
        g_solve.level_of_last = __ldcg(&st->level_of_last);
    }
}

// Threads 0..31 write g_solve's state and last outputs to `st`.
__device__ __forceinline__ void publish_solve(GNState *st) {
    const int t = (int)threadIdx.x;
    if (t >= 32) return;
    if (t < 12) {
        st->est[t] = g_solve.est[t];
        st->best[t] = g_solve.best[t];
        st->Tf[t] = g_solve.Tf[t];
    }
    for (int k = t; k < 36; k += 32) st->H[k] = g_solve.H[k];
    if (t < 6) {
        st->b[t] = g_solve.b[t];
        st->last_update[t] = g_solve.last_update[t];
    }
    if (t < 4) st->stats[t] = g_solve.stats[t];
    if (t == 0) {
        st->last_error = g_solve.last_error;
        st->n_success = g_solve.n_success;
        st->n_iter = g_solve.n_iter;
        st->failed = g_solve.failed;
        st->level_of_last = g_solve.level_of_last;
        st->huber_th = g_solve.huber_th;
    }
}

}  // namespace yas
