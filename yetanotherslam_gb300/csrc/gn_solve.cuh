// gn_solve.cuh — the FP64 solve of one Gauss-Newton iteration (GetTransform's
// loop body, RGBDFusion/src/RGBDTracking.cu:184-207), run by the 32 lanes of
// one warp on inputs and outputs in the CTA's shared memory.
//
// Semantics:
//   H = H_rgb + 100 H_icp, b = b_rgb + 10 b_icp (RGBDTracking.cu:543-544);
//   error = sqrt(residualSum) / (numResidual + 6), in FP32 as the reference;
//   update = LDLT(H).solve(b) in FP64: LDL^T with diagonal pivoting (largest
//   remaining |diagonal|, first on ties, a NaN never chosen), pseudo-inverse
//   of D (|d| <= 1/DBL_MAX -> 0), identity transpositions and no factorisation
//   if the first pivot is zero, L columns of later zero pivots left undivided
//   (Eigen 3's LDLT);
//   NaN in update(0): the iteration fails and the result is the identity;
//   estimate = exp(update) * estimate (SE(3) exponential, FP64);
//   the kept estimate is the one after an update whose error (measured before
//   the update) beat the level's best so far.
//
// GB300 executes one FP64 warp instruction per ~64 cycles per scheduler, with
// or without dependencies, so the cost of the solve is its count of FP64 warp
// instructions.  The layout minimises that count: lane 0..20 holds one element
// (i, j), j <= i, of the lower triangle of H, lanes 21..26 hold b, so one
// elimination step is four FP64 instructions for the whole trailing matrix
// and b; pivot tests, NaN tests and reciprocal seeds are integer bit
// operations; the SE(3) exponential computes its three series on three lanes
// and one entry of [R | t] per lane.
#pragma once

#include <cfloat>

#include "yas_track.h"

namespace yas {

// Packed index k of the 28 products of [J | r]: rows i, columns j >= i
// (RankUpdateHessian<6,7>, TrackingUtils.h:45-58).
__device__ __forceinline__ int pack_index(int r, int c) { return 7 * r - (r * (r - 1)) / 2 + c - r; }

// Taylor coefficients (in th^2) of sin(th)/th, (1-cos th)/th^2, (th-sin th)/th^3.
__constant__ double c_exp_poly[3][5] = {
    {1.0, -1.0 / 6.0, 1.0 / 120.0, -1.0 / 5040.0, 1.0 / 362880.0},
    {0.5, -1.0 / 24.0, 1.0 / 720.0, -1.0 / 40320.0, 1.0 / 3628800.0},
    {1.0 / 6.0, -1.0 / 120.0, 1.0 / 5040.0, -1.0 / 362880.0, 1.0 / 39916800.0}};

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
        while (tri_lane(ei + 1, 0) <= lane) ++ei;
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
    const double residualSum = (double)(float)(mode == YAS_TRACK_RGB ? S.B[27] : S.A[27]);
    const double numResidual = (double)(float)(mode == YAS_TRACK_ICP ? S.A[28] : S.A[29]);
    if (lane == 0) {
        S.stats[0] = residualSum;
        S.stats[1] = numResidual;
        S.stats[2] = (double)S.huber_th;
        S.stats[3] = S.A[28];
    }
    if (no_update) {
        __syncwarp();
        return;
    }
    const float error = sqrtf((float)residualSum) / ((float)numResidual + 6.0f);
    // ---- right-looking LDL^T with diagonal pivoting on [H | b]
    int orig = ei;  // b lanes: original index of the row they hold
    bool broke = false;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        // pivot: largest |diagonal| over k..5, first on ties; a NaN never wins
        // and a NaN at k keeps k; |doubles| order like their bit patterns
        const unsigned long long ab = abs_bits(a);
        const long long key = (ism && ei == ej) ? (ab > kInfBits ? -1LL : (long long)ab) : -2LL;
        long long kq[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) kq[q] = __shfl_sync(kAll, key, tri_lane(q, q));
        int p = k;
        if (kq[k] >= 0) {
            long long bestk = kq[k];
#pragma unroll
            for (int q = k + 1; q < 6; ++q)
                if (kq[q] > bestk) {
                    bestk = kq[q];
                    p = q;
                }
        }
        if (p != k) {
            // symmetric swap of k and p: element (i, j) <- (pi(i), pi(j))
            const int si = ei == k ? p : (ei == p ? k : ei);
            const int sj = ej == k ? p : (ej == p ? k : ej);
            const int src = ism ? (si >= sj ? tri_lane(si, sj) : tri_lane(sj, si)) : (isb ? 21 + si : lane);
            a = __shfl_sync(kAll, a, src);
            orig = __shfl_sync(kAll, orig, src);
        }
        const double d = __shfl_sync(kAll, a, tri_lane(k, k));
        const unsigned long long db = abs_bits(d);
        const bool valid = db != 0ull && db <= kInfBits;
        if (k == 0 && !valid) {
            broke = true;  // identity transpositions, the matrix is used as it is
            break;
        }
        // l_ik = a_ik / d on the column-k lanes (undivided for a zero pivot)
        const double l = valid ? div_seeded(a, d) : a;
        const bool colk = ism && ej == k && ei > k;
        // trailing update a_ij -= l_ik a_jk (i >= j > k), b_i -= l_ik b_k (i > k)
        int src_l = lane, src_x = lane;
        const bool upd = ei > k && ((ism && ej > k && valid) || isb);
        if (upd) {
            src_l = tri_lane(ei, k);
            src_x = isb ? 21 + k : tri_lane(ej, k);
        }
        const double lik = __shfl_sync(kAll, l, src_l);
        const double ajk = __shfl_sync(kAll, a, src_x);
        const double na = fma(-lik, ajk, a);
        if (upd) a = na;
        if (colk) a = l;
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
        // Taylor series in th^2 to the th^8 term (truncation below 3e-18); lane
        // r % 3 evaluates series r % 3
        const int sr = lane % 3;
        const double pc = fma(th2, fma(th2, fma(th2, fma(th2, c_exp_poly[sr][4], c_exp_poly[sr][3]), c_exp_poly[sr][2]),
                                       c_exp_poly[sr][1]),
                              c_exp_poly[sr][0]);
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
