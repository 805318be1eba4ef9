// tracker.cu — coarse-to-fine dense RGB-D tracker (photometric + point-to-plane
// ICP), with the per-pixel residual/Jacobian passes, the J^T J / J^T r
// reductions and the FP64 6x6 solve + SE(3) update all on the device.
//
// Reference semantics (paths relative to the reference project root):
//   GetTransform          RGBDFusion/src/RGBDTracking.cu:152-214: levels coarse to fine,
//                         iterations[l] per level; error = sqrt(residualSum)/(n + 6);
//                         update = LDLT(H).solve(b) in FP64; NaN in update(0) aborts with
//                         the identity; estimate = exp(update) * estimate; the returned
//                         pose is the last estimate produced by an iteration whose error
//                         (measured before its update) beat the level's best.
//   photometric step      RGBDTracking.cu:225-292, RGBDFusion/include/TrackingUtils.h:73-220,
//                         578-607: reference points warped by T with the reference inverse
//                         depth, bilinear current intensity/gradients, residual
//                         I_cur - I_ref, valid if |grad| > 0 and finite; Huber-style weight
//                         th/|r| with th = 4.685 * stddev; row [J | -r].
//   ICP step              RGBDTracking.cu:305-441: model vertex/normal moved by T, projected
//                         with round-to-nearest into the current maps; accepted when
//                         |n_c x n_m| < sin 20 deg, |v_m - v_c| <= 0.01 m and both normals
//                         valid; row [n, v x n | n.(v_c - v_m)].
//   combination           RGBDTracking.cu:521-545: H = H_rgb + 100 H_icp, b = b_rgb + 10 b_icp.
//   28-term layout        TrackingUtils.h:45-58 (RankUpdateHessian<6,7>).
//
// GB300 design: pass A fuses the reference-point warp, the photometric residual
// (with sum r, sum r^2 and the count for the variance) and the complete ICP
// products in one read of the maps; pass B forms the weighted photometric
// products.  Each pass reduces 32 values per CTA with a 31-shuffle transpose
// reduction, writes one FP64 row per CTA, and the last CTA to finish (ticket
// counter, no waiting) sums the rows in a fixed order in FP64 and, after the
// final pass, solves and updates the pose in FP64.  Nothing returns to the
// host between iterations, so a whole frame can be captured in a CUDA graph.
// Per-thread sums cover at most 4 pixels before the pairwise tree, so the FP32
// part of every reduction is pairwise.
#include <cfloat>
#include <cstring>

#include "yas_track.h"

namespace yas {

struct PassArgs {
    LevelCam c;
    int level;
    int mode;
    int first_of_level;
    int no_update;
    int L;
    float angle_th, dist_th;
    const float *ref_int;
    const float *ref_invd;
    const float4 *ref_vmap;
    const float4 *ref_nmap;
    const float *cur_int;
    const float *cur_gx;
    const float *cur_gy;
    const float4 *cur_vmap;
    const float4 *cur_nmap;
    float4 *res4;
    float *partial;
    float *grow;
    unsigned *counter;
    GNState *st;
    double Kd[kMaxLevels][4];
};

// ---------------------------------------------------------------- reductions
// Sums v[0..31] over the warp in 31 shuffles; lane L returns the sum of v[L].
__device__ __forceinline__ float warp_transpose_reduce(float v[32]) {
    const unsigned lane = lane_id();
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < off; ++i) {
            float send = upper ? v[i] : v[i + off];
            float keep = upper ? v[i + off] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    return v[0];
}

// Error-free transformation of a + b (Knuth's TwoSum): a + b == s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// CTA reduction of 32 values, then the grid totals by a two-level tree of
// "last CTA to finish" reducers (ticket counters, nobody waits):
//   * per CTA: warp transpose reduction and an 8-way cross-warp sum
//     (pairwise, FP32) give one FP32 row per CTA;
//   * per group of kGroup CTAs: the group's last CTA folds its rows with
//     compensated FP32 (TwoSum) into a (hi, lo) row;
//   * grid: the last group reducer folds the group rows the same way in
//     eight interleaved subsets and adds the eight subset sums in FP64.
// Every level is one batch of independent loads, and the order is fixed, so
// results are reproducible.  Returns true in the final CTA, where tot[0..31]
// (shared) holds the totals.  counters[0] is the grid ticket, counters[1+g]
// the ticket of group g; each is reset by the CTA that consumes it.
constexpr unsigned kGroup = 32;

__device__ __forceinline__ bool grid_reduce32(float v[32], float *partial, float *grow, unsigned *counters,
                                              double *tot) {
    constexpr unsigned S = kTrackThreads / 32;  // subsets (= warps)
    __shared__ float wsum[S][32];
    __shared__ float lsum[S][32];
    __shared__ double dsum[S][32];
    __shared__ bool flag;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const unsigned c = threadIdx.x & 31, sub = threadIdx.x >> 5;
    float r = warp_transpose_reduce(v);
    wsum[warp][lane] = r;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = 0.0f;
#pragma unroll
        for (unsigned w = 0; w < S; ++w) s += wsum[w][threadIdx.x];
        partial[blockIdx.x * 32 + threadIdx.x] = s;
        __threadfence();
    }
    __syncthreads();
    const unsigned g = blockIdx.x / kGroup;
    const unsigned g0 = g * kGroup;
    const unsigned gsize = min(kGroup, gridDim.x - g0);
    const unsigned ngroups = (gridDim.x + kGroup - 1) / kGroup;
    if (threadIdx.x == 0) flag = (atomicAdd(&counters[1 + g], 1u) == gsize - 1);
    __syncthreads();
    if (!flag) return false;
    __threadfence();
    {  // group level: subset `sub` folds rows g0 + sub + S*q
        float h = 0.0f, l = 0.0f, x[kGroup / S];
#pragma unroll
        for (unsigned q = 0; q < kGroup / S; ++q) {
            const unsigned row = sub + S * q;
            x[q] = row < gsize ? __ldcg(partial + (g0 + row) * 32 + c) : 0.0f;
        }
#pragma unroll
        for (unsigned q = 0; q < kGroup / S; ++q) {
            float s, e;
            two_sum(h, x[q], s, e);
            h = s;
            l += e;
        }
        wsum[sub][c] = h;
        lsum[sub][c] = l;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        float h = wsum[0][c], l = lsum[0][c];
#pragma unroll
        for (unsigned k = 1; k < S; ++k) {
            float s, e;
            two_sum(h, wsum[k][c], s, e);
            h = s;
            l += e + lsum[k][c];
        }
        grow[g * 64 + c] = h;
        grow[g * 64 + 32 + c] = l;
        __threadfence();
    }
    if (threadIdx.x == 0) counters[1 + g] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) flag = (atomicAdd(&counters[0], 1u) == ngroups - 1);
    __syncthreads();
    if (!flag) return false;
    __threadfence();
    {  // grid level: subset `sub` folds group rows sub, sub + S, ...
        float h = 0.0f, l = 0.0f;
        for (unsigned row = sub; row < ngroups; row += 2 * S) {
            const float xh0 = __ldcg(grow + row * 64 + c), xl0 = __ldcg(grow + row * 64 + 32 + c);
            const bool two = row + S < ngroups;
            const float xh1 = two ? __ldcg(grow + (row + S) * 64 + c) : 0.0f;
            const float xl1 = two ? __ldcg(grow + (row + S) * 64 + 32 + c) : 0.0f;
            float s, e;
            two_sum(h, xh0, s, e);
            h = s;
            l += e + xl0;
            two_sum(h, xh1, s, e);
            h = s;
            l += e + xl1;
        }
        dsum[sub][c] = (double)h + (double)l;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = 0.0;
#pragma unroll
        for (unsigned k = 0; k < S; ++k) s += dsum[k][threadIdx.x];
        tot[threadIdx.x] = s;
    }
    if (threadIdx.x == 0) counters[0] = 0u;
    __syncthreads();
    return true;
}

// ---------------------------------------------------------------- FP64 algebra
// FP64 on GB300 has a dependent latency of about 65 cycles (16x FP32) and an
// IEEE FP64 division is a multi-step sequence; the solve therefore avoids
// divisions (FP32-seeded reciprocals, polynomial series for small angles).

// Float copy of the estimate read by the pixel passes.
__device__ void publish_estimate(GNState *st, const double Kd[kMaxLevels][4], int L) {
    (void)Kd;
    (void)L;
    const double *E = st->est;
    for (int i = 0; i < 12; ++i) st->Tf[i] = (float)E[i];
}

// R * K_l^-1 for TransformReferencePoint (ImageProc.cu:86-101), formed in FP32
// from the FP32 estimate by each CTA (the reference forms it in FP64 and
// rounds it to FP32; the two differ by an ulp).
__device__ __forceinline__ void make_rkinv(const float *T, const LevelCam &c, float *RK) {
    const float cxi = c.cx * c.invfx, cyi = c.cy * c.invfy;
    for (int i = 0; i < 3; ++i) {
        RK[i * 3 + 0] = T[i * 4 + 0] * c.invfx;
        RK[i * 3 + 1] = T[i * 4 + 1] * c.invfy;
        RK[i * 3 + 2] = T[i * 4 + 2] - T[i * 4 + 0] * cxi - T[i * 4 + 1] * cyi;
    }
}

// Packed index k of the 28 products of [J | r]: rows i, columns j >= i
// (RankUpdateHessian<6,7>, TrackingUtils.h:45-58).
__constant__ signed char c_pack_i[27] = {0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 5, 5};
// Taylor coefficients (in th^2) of sin(th)/th, (1-cos th)/th^2, (th-sin th)/th^3.
__constant__ double c_exp_poly[3][5] = {
    {1.0, -1.0 / 6.0, 1.0 / 120.0, -1.0 / 5040.0, 1.0 / 362880.0},
    {0.5, -1.0 / 24.0, 1.0 / 720.0, -1.0 / 40320.0, 1.0 / 3628800.0},
    {1.0 / 6.0, -1.0 / 120.0, 1.0 / 5040.0, -1.0 / 362880.0, 1.0 / 39916800.0}};
__constant__ signed char c_pack_j[27] = {0, 1, 2, 3, 4, 5, 6, 1, 2, 3, 4, 5, 6, 2, 3, 4, 5, 6, 3, 4, 5, 6, 4, 5, 6, 5, 6};

// Reciprocal for the solve: FP32 seed and one Newton step in FP64 (relative
// error below 2^-46, far under the ~1e-7 precision of the FP32-accumulated
// system it is applied to).
__device__ __forceinline__ double drcp1(double d) {
    const double ad = fabs(d);
    if (!(ad > 1e-30 && ad < 1e30)) return 1.0 / d;
    const double r = (double)__frcp_rn((float)d);
    return fma(r, fma(-d, r, 1.0), r);
}

__device__ __forceinline__ int pack_index(int r, int c) { return 7 * r - (r * (r - 1)) / 2 + c - r; }

// The solve of one Gauss-Newton iteration, executed by the 32 lanes of warp 0
// of the final CTA (GetTransform's loop body, RGBDTracking.cu:184-207):
//   H = H_rgb + 100 H_icp, b = b_rgb + 10 b_icp (RGBDTracking.cu:543-544);
//   error = sqrt(residualSum) / (numResidual + 6), in FP32 as the reference;
//   update = LDLT(H).solve(b) in FP64: LDL^T with diagonal pivoting (largest
//   remaining diagonal, first on ties, left-looking), pseudo-inverse of D
//   (|d| <= 1/DBL_MAX -> 0), identity transpositions and no factorisation if
//   the first pivot is zero (Eigen 3's LDLT);
//   NaN in update(0): the iteration fails and the result is the identity;
//   estimate = exp(update) * estimate (SE(3) exponential, FP64);
//   the kept estimate is the one after an update whose error beat the level's.
// GB300's dependent FP64 latency is ~65 cycles, so the solve keeps row i of H
// in the registers of lane i, moves columns between lanes with shuffles, runs
// every independent FP64 product on its own lane, and unrolls the
// factorisation so that every register index is static.
__device__ __noinline__ void gn_solve_warp(const PassArgs &a) {
    __shared__ double Ls[36];
    GNState *st = a.st;
    const int lane = (int)(threadIdx.x & 31);
    const double *A = st->a_sums, *B = st->b_sums;
    const bool rowlane = lane < 6;
    // ---- assemble row `lane` of H and b[lane]
    double row[6], y = 0.0;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        row[j] = 0.0;
        if (rowlane) {
            const int kk = pack_index(min(lane, j), max(lane, j));
            row[j] = a.mode == YAS_TRACK_RGBD ? fma(100.0, A[kk], B[kk]) : (a.mode == YAS_TRACK_RGB ? B[kk] : A[kk]);
        }
    }
    if (rowlane) {
        const int kk = pack_index(lane, 6);
        y = a.mode == YAS_TRACK_RGBD ? fma(10.0, A[kk], B[kk]) : (a.mode == YAS_TRACK_RGB ? B[kk] : A[kk]);
#pragma unroll
        for (int j = 0; j < 6; ++j) st->H[lane * 6 + j] = row[j];
        st->b[lane] = y;
    }
    const double residualSum = (double)(float)(a.mode == YAS_TRACK_RGB ? B[27] : A[27]);
    const double numResidual = (double)(float)(a.mode == YAS_TRACK_ICP ? A[28] : A[29]);
    if (lane == 0) {
        st->stats[0] = residualSum;
        st->stats[1] = numResidual;
        st->stats[2] = st->huber_th;
        st->stats[3] = A[28];
    }
    if (a.no_update) return;
    const float error = sqrtf((float)residualSum) / ((float)numResidual + 6.0f);
    // ---- LDL^T with diagonal pivoting
    double Dv[6];
    int trk[6];
    bool broke = false;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        Dv[k] = 0.0;
        trk[k] = k;
        if (broke) continue;
        // pivot: largest |diagonal| over rows k..5, first one on ties; a NaN
        // never wins (every comparison with it is false) and a NaN at row k
        // keeps row k; non-negative doubles order like their bit patterns
        double diag = 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q)
            if (lane == q) diag = row[q];
        long long key = (lane >= k && lane < 6) ? (isnan(diag) ? -1LL : __double_as_longlong(fabs(diag))) : -2LL;
        const long long keyk = __shfl_sync(0xffffffffu, key, k);
        int p = k;
        if (keyk >= 0) {
            long long bk = key;
            int bl = lane;
#pragma unroll
            for (int off = 1; off < 8; off <<= 1) {
                const long long ok = __shfl_xor_sync(0xffffffffu, bk, off);
                const int ol = __shfl_xor_sync(0xffffffffu, bl, off);
                if (ok > bk || (ok == bk && ol < bl)) {
                    bk = ok;
                    bl = ol;
                }
            }
            p = __shfl_sync(0xffffffffu, bl, 0);
        }
        trk[k] = p;
        if (p != k) {
            // rows k and p change lanes, then every row swaps columns k and p
            const int src = lane == k ? p : (lane == p ? k : lane);
#pragma unroll
            for (int q = 0; q < 6; ++q) row[q] = __shfl_sync(0xffffffffu, row[q], src);
#pragma unroll
            for (int q = k + 1; q < 6; ++q)
                if (q == p) {
                    const double t = row[k];
                    row[k] = row[q];
                    row[q] = t;
                }
        }
        if (k > 0) {
            double tmp[6];
#pragma unroll
            for (int j = 0; j < k; ++j) tmp[j] = Dv[j] * __shfl_sync(0xffffffffu, row[j], k);
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < k; ++j) s = fma(row[j], tmp[j], s);
            if (lane >= k) row[k] -= s;
        }
        const double d = __shfl_sync(0xffffffffu, row[k], k);
        Dv[k] = d;
        const bool valid = fabs(d) > 0.0;
        if (k == 0 && !valid) {
            broke = true;  // identity transpositions, the matrix is used as it is
            continue;
        }
        if (valid && lane > k) row[k] *= drcp1(d);
    }
    // ---- y = P b; L y' = y; D y'' = y'; L^T x = y''; x = P^T x
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int p = trk[k];
        const int src = lane == k ? p : (lane == p ? k : lane);
        y = __shfl_sync(0xffffffffu, y, src);
    }
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const double yj = __shfl_sync(0xffffffffu, y, j);
        if (lane > j && rowlane) y = fma(-row[j], yj, y);
    }
    {
        double dd = 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q)
            if (lane == q) dd = row[q];
        y = (rowlane && fabs(dd) > 1.0 / DBL_MAX) ? y * drcp1(dd) : 0.0;
    }
    if (rowlane) {
#pragma unroll
        for (int q = 0; q < 6; ++q) Ls[lane * 6 + q] = row[q];
    }
    __syncwarp();
#pragma unroll
    for (int j = 5; j > 0; --j) {
        const double yj = __shfl_sync(0xffffffffu, y, j);
        const double lji = rowlane ? Ls[j * 6 + lane] : 0.0;  // L(j, lane)
        if (lane < j) y = fma(-lji, yj, y);
    }
#pragma unroll
    for (int k = 5; k >= 0; --k) {
        const int p = trk[k];
        const int src = lane == k ? p : (lane == p ? k : lane);
        y = __shfl_sync(0xffffffffu, y, src);
    }
    double u[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) u[q] = __shfl_sync(0xffffffffu, y, q);
    if (lane < 6) st->last_update[lane] = y;
    if (isnan(u[0])) {
        if (lane == 0) st->failed = 1;
        if (lane < 12) st->best[lane] = (lane % 5 == 0) ? 1.0 : 0.0;
        return;
    }
    // ---- SE(3) exponential, one matrix entry per lane:
    // R = I + A W + B W^2, t = V v, V = I + B W + C W^2, W = hat(w),
    // W^2 = w w^T - th^2 I, W v = w x v
    const double wx = u[3], wy = u[4], wz = u[5];
    const double th2 = fma(wx, wx, fma(wy, wy, wz * wz));
    double cA, cB, cC;
    if (th2 < 1e-2) {
        // Taylor series in th^2 to the th^8 term (truncation below 3e-18)
        cA = fma(th2, fma(th2, fma(th2, fma(th2, c_exp_poly[0][4], c_exp_poly[0][3]), c_exp_poly[0][2]), c_exp_poly[0][1]),
                 c_exp_poly[0][0]);
        cB = fma(th2, fma(th2, fma(th2, fma(th2, c_exp_poly[1][4], c_exp_poly[1][3]), c_exp_poly[1][2]), c_exp_poly[1][1]),
                 c_exp_poly[1][0]);
        cC = fma(th2, fma(th2, fma(th2, fma(th2, c_exp_poly[2][4], c_exp_poly[2][3]), c_exp_poly[2][2]), c_exp_poly[2][1]),
                 c_exp_poly[2][0]);
    } else {
        const double th = sqrt(th2);
        double sn, cs;
        sincos(th, &sn, &cs);
        cA = sn / th;
        cB = (1.0 - cs) / th2;
        cC = (th - sn) / (th2 * th);
    }
    const double w[3] = {wx, wy, wz};
    const int i = (lane < 12) ? lane / 4 : 0, jc = (lane < 12) ? lane % 4 : 0;
    // row i of E: E(i,q) = d(i,q) + A W(i,q) + B (w_i w_q - d(i,q) th^2)
    double Er[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double Wiq = (i == q) ? 0.0
                                    : ((i == 0 && q == 1) ? -wz
                                       : (i == 0 && q == 2) ? wy
                                       : (i == 1 && q == 0) ? wz
                                       : (i == 1 && q == 2) ? -wx
                                       : (i == 2 && q == 0) ? -wy
                                                            : wx);
        const double dq = (i == q) ? 1.0 : 0.0;
        Er[q] = fma(cA, Wiq, fma(cB, fma(w[i], w[q], -dq * th2), dq));
    }
    // t_i = v_i + B (w x v)_i + C (w_i (w . v) - th^2 v_i)
    const double wxv[3] = {wy * u[2] - wz * u[1], wz * u[0] - wx * u[2], wx * u[1] - wy * u[0]};
    const double wdv = fma(wx, u[0], fma(wy, u[1], wz * u[2]));
    const double ti = fma(cB, wxv[i], fma(cC, fma(w[i], wdv, -th2 * u[i]), u[i]));
    // ---- estimate = E * estimate, entry (i, jc) on lane i*4 + jc
    double o = 0.0;
    if (lane < 12) {
        const double e0 = st->est[0 * 4 + jc], e1 = st->est[1 * 4 + jc], e2 = st->est[2 * 4 + jc];
        o = fma(Er[0], e0, fma(Er[1], e1, Er[2] * e2));
        if (jc == 3) o += ti;
    }
    __syncwarp();
    if (lane < 12) {
        st->est[lane] = o;
        st->Tf[lane] = (float)o;
    }
    // ---- acceptance on the error measured before the update
    int accept = 0;
    if (lane == 0) {
        if (a.first_of_level) st->last_error = (double)FLT_MAX;
        accept = (double)error < st->last_error;
        if (accept) {
            st->last_error = (double)error;
            st->n_success++;
        }
        st->n_iter++;
        st->level_of_last = a.level;
    }
    accept = __shfl_sync(0xffffffffu, accept, 0);
    if (accept && lane < 12) st->best[lane] = o;
}

// ---------------------------------------------------------------- pixel math
// TransformReferencePoint (ImageProc.cu:42-78): (RKinv (x,y,1)) z + t, fixed order.
__device__ __forceinline__ float3 warp_ref_point(const float *RK, const float *T, int x, int y, float z) {
    const float fx = (float)x, fy = (float)y;
    float3 p;
    p.x = __fadd_rn(__fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(RK[0], fx), __fmul_rn(RK[1], fy)), RK[2]), z), T[3]);
    p.y = __fadd_rn(__fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(RK[3], fx), __fmul_rn(RK[4], fy)), RK[5]), z), T[7]);
    p.z = __fadd_rn(__fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(RK[6], fx), __fmul_rn(RK[7], fy)), RK[8]), z), T[11]);
    return p;
}

__device__ __forceinline__ float bilinear(const float *__restrict__ m, int w, float x, float y) {
    const int u = (int)floorf(x), v = (int)floorf(y);
    const float cx = x - (float)u, cy = y - (float)v;
    const float *r0 = m + (size_t)v * w + u, *r1 = r0 + w;
    return (__ldg(r0) * (1.0f - cx) + __ldg(r0 + 1) * cx) * (1.0f - cy) +
           (__ldg(r1) * (1.0f - cx) + __ldg(r1 + 1) * cx) * cy;
}

__global__ void __launch_bounds__(kTrackThreads, 4) gn_pass_a(PassArgs a) {
    GNState *st = a.st;
    if (*(volatile int *)&st->failed) return;
    __shared__ float sT[12], sRK[9];
    __shared__ double tot[32];
    if (threadIdx.x < 12) sT[threadIdx.x] = st->Tf[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) make_rkinv(sT, a.c, sRK);
    __syncthreads();
    const LevelCam c = a.c;
    const int n = c.w * c.h;
    float acc[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) acc[i] = 0.0f;
    const bool do_rgb = (a.mode & YAS_TRACK_RGB) != 0, do_icp = (a.mode & YAS_TRACK_ICP) != 0;
    for (int k = blockIdx.x * kTrackThreads + threadIdx.x; k < n; k += gridDim.x * kTrackThreads) {
        const int y = k / c.w, x = k - y * c.w;
        if (do_rgb) {
            float r = 0.0f, gx = 0.0f, gy = 0.0f;
            bool ok = false;
            const float zinv = __ldg(a.ref_invd + k);
            if (zinv > 0.0f) {
                const float z = 1.0f / zinv;
                const float3 p = warp_ref_point(sRK, sT, x, y, z);
                const float u = c.fx * p.x / p.z + c.cx;
                const float v = c.fy * p.y / p.z + c.cy;
                if (u > 0.0f && v > 0.0f && u < (float)(c.w - 1) && v < (float)(c.h - 1)) {
                    r = bilinear(a.cur_int, c.w, u, v) - __ldg(a.ref_int + k);
                    gx = bilinear(a.cur_gx, c.w, u, v);
                    gy = bilinear(a.cur_gy, c.w, u, v);
                    ok = (gx * gx + gy * gy) > 0.0f && isfinite(r);
                }
            }
            a.res4[k] = make_float4(r, gx, gy, ok ? 1.0f : -1.0f);
            if (ok) {
                acc[29] += 1.0f;
                acc[30] += r;
                acc[31] += r * r;
            }
        }
        if (do_icp) {
            const float4 vm = __ldg(a.ref_vmap + k);
            if (vm.w >= 0.0f) {
                const float3 vl = make_float3(sT[0] * vm.x + sT[1] * vm.y + sT[2] * vm.z + sT[3],
                                              sT[4] * vm.x + sT[5] * vm.y + sT[6] * vm.z + sT[7],
                                              sT[8] * vm.x + sT[9] * vm.y + sT[10] * vm.z + sT[11]);
                const float invz = 1.0f / vl.z;
                const int u = (int)floorf(c.fx * vl.x * invz + c.cx + 0.5f);
                const int v = (int)floorf(c.fy * vl.y * invz + c.cy + 0.5f);
                if (u >= 0 && v >= 0 && u < c.w && v < c.h) {
                    const float4 vc = __ldg(a.cur_vmap + v * c.w + u);
                    if (vc.w >= 0.0f) {
                        const float4 nm = __ldg(a.ref_nmap + k);
                        const float3 nl = make_float3(sT[0] * nm.x + sT[1] * nm.y + sT[2] * nm.z,
                                                      sT[4] * nm.x + sT[5] * nm.y + sT[6] * nm.z,
                                                      sT[8] * nm.x + sT[9] * nm.y + sT[10] * nm.z);
                        const float4 nc = __ldg(a.cur_nmap + v * c.w + u);
                        const float dx = vl.x - vc.x, dy = vl.y - vc.y, dz = vl.z - vc.z;
                        const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
                        const float cx_ = nc.y * nl.z - nc.z * nl.y, cy_ = nc.z * nl.x - nc.x * nl.z,
                                    cz_ = nc.x * nl.y - nc.y * nl.x;
                        const float angle = sqrtf(cx_ * cx_ + cy_ * cy_ + cz_ * cz_);
                        if (angle < a.angle_th && dist <= a.dist_th && nm.w > 0.0f && nc.w > 0.0f) {
                            float row[7];
                            row[0] = nl.x;
                            row[1] = nl.y;
                            row[2] = nl.z;
                            row[3] = vl.y * nl.z - vl.z * nl.y;
                            row[4] = vl.z * nl.x - vl.x * nl.z;
                            row[5] = vl.x * nl.y - vl.y * nl.x;
                            row[6] = nl.x * (vc.x - vl.x) + nl.y * (vc.y - vl.y) + nl.z * (vc.z - vl.z);
                            int q = 0;
#pragma unroll
                            for (int i = 0; i < 7; ++i)
#pragma unroll
                                for (int j = i; j < 7; ++j) acc[q++] += row[i] * row[j];
                            acc[28] += 1.0f;
                        }
                    }
                }
            }
        }
    }
    if (!grid_reduce32(acc, a.partial, a.grow, a.counter, tot)) return;
    if (threadIdx.x < 32) st->a_sums[threadIdx.x] = tot[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {
        // Huber threshold 4.685 * stddev of the photometric residuals, in FP32
        // as the reference (RGBDTracking.cu:259-278): mean = sum r / n, then
        // sum (r - mean)^2 = sum r^2 - 2 mean sum r + n mean^2 from the FP64
        // totals (the reference's second pass over the residuals).
        const double nn = tot[29], s = tot[30], s2 = tot[31];
        const float mean = (float)s / (float)nn;
        const double md = (double)mean;
        const double ss = fma(nn * md, md, fma(-2.0 * md, s, s2));
        const float var = sqrtf((float)ss / ((float)nn - 1.0f));
        st->huber_th = (float)(4.685 * (double)var);
    }
    if (a.mode == YAS_TRACK_ICP) {
        __syncthreads();
        if (threadIdx.x < 32) gn_solve_warp(a);
    }
}

__global__ void __launch_bounds__(kTrackThreads, 4) gn_pass_b(PassArgs a) {
    GNState *st = a.st;
    if (*(volatile int *)&st->failed) return;
    __shared__ float sT[12], sRK[9];
    __shared__ double tot[32];
    if (threadIdx.x < 12) sT[threadIdx.x] = st->Tf[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) make_rkinv(sT, a.c, sRK);
    __syncthreads();
    const float th = st->huber_th;
    const LevelCam c = a.c;
    const int n = c.w * c.h;
    float acc[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) acc[i] = 0.0f;
    for (int k = blockIdx.x * kTrackThreads + threadIdx.x; k < n; k += gridDim.x * kTrackThreads) {
        const float4 res = a.res4[k];
        if (res.w > 0.0f) {
            const int y = k / c.w, x = k - y * c.w;
            const float z = 1.0f / __ldg(a.ref_invd + k);
            const float3 p = warp_ref_point(sRK, sT, x, y, z);
            const float zInv = 1.0f / p.z;
            float wt = 1.0f;
            if (fabsf(res.x) > th) wt = th / fabsf(res.x);
            float row[7];
            row[0] = res.y * c.fx * zInv;
            row[1] = res.z * c.fy * zInv;
            row[2] = -(row[0] * p.x + row[1] * p.y) * zInv;
            row[3] = row[2] * p.y - res.z * c.fy;
            row[4] = -row[2] * p.x + res.y * c.fx;
            row[5] = -row[0] * p.y + row[1] * p.x;
            row[6] = -res.x;
            int q = 0;
#pragma unroll
            for (int i = 0; i < 7; ++i)
#pragma unroll
                for (int j = i; j < 7; ++j) acc[q++] += wt * row[i] * row[j];
        }
    }
    if (!grid_reduce32(acc, a.partial, a.grow, a.counter, tot)) return;
    if (threadIdx.x < 32) st->b_sums[threadIdx.x] = tot[threadIdx.x];
    __syncthreads();
    if (threadIdx.x < 32) gn_solve_warp(a);
}

__global__ void gn_init_kernel(GNState *st, Pose64 init, int L, PassArgs kargs) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) st->est[i * 4 + j] = init.r[i * 3 + j];
        st->est[i * 4 + 3] = init.t[i];
    }
    for (int i = 0; i < 12; ++i) st->best[i] = st->est[i];
    st->last_error = (double)FLT_MAX;
    st->failed = 0;
    st->n_iter = 0;
    st->n_success = 0;
    st->level_of_last = -1;
    publish_estimate(st, kargs.Kd, L);
}

// ---------------------------------------------------------------- host side
static PassArgs make_args(yas_tracker *tr, int l, int first, int no_update) {
    PassArgs a;
    memset(&a, 0, sizeof(a));
    a.c = tr->cam[l];
    a.level = l;
    a.mode = tr->mode;
    a.first_of_level = first;
    a.no_update = no_update;
    a.L = tr->L;
    a.angle_th = tr->angle_th;
    a.dist_th = tr->dist_th;
    TrackLevelBufs &cb = tr->curb(l), &rb = tr->refb(l);
    a.ref_int = rb.intensity;
    a.ref_invd = rb.invd;
    a.ref_vmap = rb.vmap;
    a.ref_nmap = rb.nmap;
    a.cur_int = cb.intensity;
    a.cur_gx = tr->gx[l];
    a.cur_gy = tr->gy[l];
    a.cur_vmap = cb.vmap;
    a.cur_nmap = cb.nmap;
    a.res4 = tr->res4;
    a.st = tr->state;
    for (int i = 0; i < kMaxLevels; ++i)
        for (int j = 0; j < 4; ++j) a.Kd[i][j] = tr->dK[i][j];
    return a;
}

static int pass_grid(const LevelCam &c) {
    int n = c.w * c.h;
    int g = (n + kTrackThreads * kPixPerThread - 1) / (kTrackThreads * kPixPerThread);
    return g < 1 ? 1 : (g > kMaxCtas ? kMaxCtas : g);
}

static void launch_passes(yas_tracker *tr, int l, int first, int no_update, cudaStream_t s) {
    PassArgs a = make_args(tr, l, first, no_update);
    const int g = pass_grid(tr->cam[l]);
    a.partial = tr->partialA;
    a.grow = tr->growA;
    a.counter = tr->counters;
    if (tr->hook) tr->hook(tr->hook_ctx, 10 + l);
    gn_pass_a<<<g, kTrackThreads, 0, s>>>(a);
    if (tr->mode & YAS_TRACK_RGB) {
        a.partial = tr->partialB;
        a.grow = tr->growB;
        a.counter = tr->counters + kMaxCtas / kGroup + 1;
        if (tr->hook) tr->hook(tr->hook_ctx, 20 + l);
        gn_pass_b<<<g, kTrackThreads, 0, s>>>(a);
    }
}

void launch_gn_init(yas_tracker *tr, const Pose64 &init, cudaStream_t s) {
    PassArgs a = make_args(tr, 0, 0, 0);
    gn_init_kernel<<<1, 32, 0, s>>>(tr->state, init, tr->L, a);
}

void launch_gn_iteration(yas_tracker *tr, int l, bool first_of_level, cudaStream_t s) {
    launch_passes(tr, l, first_of_level ? 1 : 0, 0, s);
}

void launch_gn_schedule(yas_tracker *tr, cudaStream_t s) {
    for (int l = tr->L - 1; l >= 0; --l)
        for (int it = 0; it < tr->iters[l]; ++it) launch_gn_iteration(tr, l, it == 0, s);
}

void launch_gn_linearise(yas_tracker *tr, int l, cudaStream_t s) { launch_passes(tr, l, 0, 1, s); }

int tracker_alloc(yas_tracker *tr) {
    auto grab = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        cudaMemset(p, 0, bytes);
        tr->allocations.push_back(p);
        return p;
    };
    for (int l = 0; l < tr->L; ++l) {
        const size_t n = (size_t)tr->cam[l].w * tr->cam[l].h;
        for (int sidx = 0; sidx < 2; ++sidx) {
            TrackLevelBufs &b = tr->set[sidx][l];
            b.intensity = (float *)grab(n * 4);
            b.invd = (float *)grab(n * 4);
            b.vmap = (float4 *)grab(n * 16);
            b.nmap = (float4 *)grab(n * 16);
            if (!b.intensity || !b.invd || !b.vmap || !b.nmap) return YAS_ERR_OOM;
        }
        tr->gx[l] = (float *)grab(n * 4);
        tr->gy[l] = (float *)grab(n * 4);
        if (!tr->gx[l] || !tr->gy[l]) return YAS_ERR_OOM;
    }
    tr->res4 = (float4 *)grab((size_t)tr->w * tr->h * 16);
    tr->partialA = (float *)grab((size_t)kMaxCtas * 32 * 4);
    tr->partialB = (float *)grab((size_t)kMaxCtas * 32 * 4);
    tr->growA = (float *)grab((size_t)(kMaxCtas / kGroup) * 64 * 4);
    tr->growB = (float *)grab((size_t)(kMaxCtas / kGroup) * 64 * 4);
    tr->counters = (unsigned *)grab((size_t)2 * (kMaxCtas / kGroup + 1) * 4);
    tr->state = (GNState *)grab(sizeof(GNState));
    tr->staging_bytes = (size_t)tr->w * tr->h * 4;
    tr->staging = grab(tr->staging_bytes);
    if (!tr->res4 || !tr->partialA || !tr->partialB || !tr->growA || !tr->growB || !tr->counters || !tr->state || !tr->staging)
        return YAS_ERR_OOM;
    if (cudaMallocHost(&tr->state_host, sizeof(GNState)) != cudaSuccess) {
        cudaGetLastError();
        return YAS_ERR_OOM;
    }
    memset(tr->state_host, 0, sizeof(GNState));
    return YAS_OK;
}

void tracker_free(yas_tracker *tr) {
    for (void *p : tr->allocations) cudaFree(p);
    tr->allocations.clear();
    if (tr->state_host) cudaFreeHost(tr->state_host);
    tr->state_host = nullptr;
}

void tracker_image(yas_tracker *tr, const uint8_t *src, int channels, int pitch, bool reference,
                   cudaStream_t s) {
    TrackLevelBufs *B = reference ? tr->set[1 - tr->cur] : tr->set[tr->cur];
    // The reference set has no gradient maps: write them to the current-frame
    // gradient buffers only when preparing the current frame.
    float *gx0 = reference ? nullptr : tr->gx[0];
    float *gy0 = reference ? nullptr : tr->gy[0];
    if (reference) {
        // gradients of a reference image are not used; compute into res4 scratch
        gx0 = reinterpret_cast<float *>(tr->res4);
        gy0 = gx0 + (size_t)tr->w * tr->h;
    }
    launch_image_level0(src, channels, 0, pitch, tr->w, tr->h, B[0].intensity, gx0, gy0, s);
    for (int l = 1; l < tr->L; ++l)
        launch_image_level(B[l - 1].intensity, tr->cam[l - 1].w, tr->cam[l - 1].h, tr->cam[l].w,
                           tr->cam[l].h, B[l].intensity, reference ? nullptr : tr->gx[l],
                           reference ? nullptr : tr->gy[l], s);
}

void tracker_depth(yas_tracker *tr, const void *src, int is_u16, int pitch, float scale, float *depth_m,
                   bool reference, cudaStream_t s) {
    TrackLevelBufs *B = reference ? tr->set[1 - tr->cur] : tr->set[tr->cur];
    launch_depth_level0(src, is_u16, pitch, scale, tr->cam[0], depth_m, B[0].invd, B[0].vmap, B[0].nmap, s);
    for (int l = 1; l < tr->L; ++l)
        launch_depth_level(B[l - 1].invd, tr->cam[l - 1].w, tr->cam[l], B[l].invd, B[l].vmap, B[l].nmap, s);
}

void tracker_model(yas_tracker *tr, cudaStream_t s) {
    TrackLevelBufs *B = tr->set[1 - tr->cur];
    launch_model_level(nullptr, 0, tr->cam[0].w, tr->cam[0].h, B[0].vmap, B[0].nmap, s);
    for (int l = 1; l < tr->L; ++l)
        launch_model_level(B[l - 1].vmap, tr->cam[l - 1].w, tr->cam[l].w, tr->cam[l].h, B[l].vmap, B[l].nmap,
                           s);
}

}  // namespace yas

// ---------------------------------------------------------------- linearisation without allocation
// yas_gn_linearise_static runs the same kernels as yas_tracker_compute_step,
// with every piece of scratch in one file-scope device array instead of
// memory allocated by a tracker handle.
namespace yas {

constexpr int kStaticMaxPixels = 640 * 480;
constexpr int kStaticMaxCtas = (kStaticMaxPixels + kTrackThreads - 1) / kTrackThreads;
constexpr int kStaticGroups = (kStaticMaxCtas + (int)kGroup - 1) / (int)kGroup;

struct StaticScratch {
    GNState state;
    float4 res4[kStaticMaxPixels];
    float partialA[kStaticMaxCtas * 32];
    float partialB[kStaticMaxCtas * 32];
    float growA[kStaticGroups * 64];
    float growB[kStaticGroups * 64];
    unsigned counters[2 * (kStaticGroups + 1)];  // pass A tickets, then pass B tickets
};

static __device__ __align__(256) StaticScratch g_static_scratch;

// Device address of g_static_scratch per device, resolved once per device.
static std::mutex g_static_mutex;
static StaticScratch *g_static_ptr[64];

static int static_scratch(StaticScratch **out) {
    int dev = 0;
    YAS_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return YAS_ERR_STATE;
    std::lock_guard<std::mutex> lk(g_static_mutex);
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        YAS_TRY_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
        g_static_ptr[dev] = static_cast<StaticScratch *>(p);
    }
    *out = g_static_ptr[dev];
    return YAS_OK;
}

__global__ void copy_linearisation(const GNState *st, double *out) {
    const int i = threadIdx.x;
    if (i < 36) out[i] = st->H[i];
    if (i < 6) out[36 + i] = st->b[i];
    if (i < 4) out[42 + i] = st->stats[i];
}

}  // namespace yas

extern "C" YAS_API int yas_gn_linearise_static(const yas_gn_level *lv, const yas_pose *T, int mode, double *dev_out,
                                               void *stream) {
    using namespace yas;
    if (!lv || !T || !dev_out) return YAS_ERR_BAD_ARG;
    if (mode != YAS_TRACK_RGB && mode != YAS_TRACK_ICP && mode != YAS_TRACK_RGBD) return YAS_ERR_BAD_ARG;
    if (lv->width < 4 || lv->height < 4 || !(lv->fx > 0.0f) || !(lv->fy > 0.0f)) return YAS_ERR_BAD_ARG;
    if ((long long)lv->width * lv->height > kStaticMaxPixels) return YAS_ERR_CAPACITY;
    if ((mode & YAS_TRACK_RGB) && (!lv->ref_intensity || !lv->ref_inv_depth || !lv->cur_intensity || !lv->cur_gx ||
                                   !lv->cur_gy))
        return YAS_ERR_BAD_ARG;
    if ((mode & YAS_TRACK_ICP) && (!lv->ref_vmap || !lv->ref_nmap || !lv->cur_vmap || !lv->cur_nmap))
        return YAS_ERR_BAD_ARG;
    StaticScratch *sc = nullptr;
    YAS_TRY(static_scratch(&sc));
    cudaStream_t s = (cudaStream_t)stream;
    // tickets must start at zero; everything else is written before it is read
    YAS_TRY_CUDA(cudaMemsetAsync(sc->counters, 0, sizeof(sc->counters), s));
    PassArgs a;
    memset(&a, 0, sizeof(a));
    a.c.fx = lv->fx;
    a.c.fy = lv->fy;
    a.c.cx = lv->cx;
    a.c.cy = lv->cy;
    a.c.invfx = (float)(1.0 / (double)lv->fx);
    a.c.invfy = (float)(1.0 / (double)lv->fy);
    a.c.w = lv->width;
    a.c.h = lv->height;
    a.level = 0;
    a.mode = mode;
    a.first_of_level = 0;
    a.no_update = 1;
    a.L = 1;
    a.angle_th = sinf(20.f * 3.14159254f / 180.f);
    a.dist_th = 0.01f;
    a.ref_int = lv->ref_intensity;
    a.ref_invd = lv->ref_inv_depth;
    a.ref_vmap = reinterpret_cast<const float4 *>(lv->ref_vmap);
    a.ref_nmap = reinterpret_cast<const float4 *>(lv->ref_nmap);
    a.cur_int = lv->cur_intensity;
    a.cur_gx = lv->cur_gx;
    a.cur_gy = lv->cur_gy;
    a.cur_vmap = reinterpret_cast<const float4 *>(lv->cur_vmap);
    a.cur_nmap = reinterpret_cast<const float4 *>(lv->cur_nmap);
    a.res4 = sc->res4;
    a.st = &sc->state;
    a.Kd[0][0] = lv->fx;
    a.Kd[0][1] = lv->fy;
    a.Kd[0][2] = lv->cx;
    a.Kd[0][3] = lv->cy;
    gn_init_kernel<<<1, 32, 0, s>>>(a.st, pose_from(*T), 1, a);
    const int g = pass_grid(a.c);
    a.partial = sc->partialA;
    a.grow = sc->growA;
    a.counter = sc->counters;
    gn_pass_a<<<g, kTrackThreads, 0, s>>>(a);
    if (mode & YAS_TRACK_RGB) {
        a.partial = sc->partialB;
        a.grow = sc->growB;
        a.counter = sc->counters + kStaticGroups + 1;
        gn_pass_b<<<g, kTrackThreads, 0, s>>>(a);
    }
    copy_linearisation<<<1, 64, 0, s>>>(a.st, dev_out);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}
