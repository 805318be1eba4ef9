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
#include <algorithm>
#include <cfloat>
#include <cstring>

#include <cuda.h>

#include "gn_solve.cuh"
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
constexpr unsigned kSubsets = kTrackThreads / 32;  // reduction subsets (= warps)

// Stage 1: the CTA's FP32 row of 32 sums, stored to `row` (visible GPU-wide
// before the function returns).
__device__ __forceinline__ void cta_row32(float v[32], float *row) {
    __shared__ float wsum[kSubsets][32];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    float r = warp_transpose_reduce(v);
    wsum[warp][lane] = r;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = 0.0f;
#pragma unroll
        for (unsigned w = 0; w < kSubsets; ++w) s += wsum[w][threadIdx.x];
        row[threadIdx.x] = s;
        __threadfence();
    }
    __syncthreads();
}

// Stage 2: CTA `cta` of `nact` takes a ticket of its group of kGroup CTAs; the
// last to arrive folds the group's rows (compensated FP32) into the (hi, lo)
// row grow[g], resets the ticket and returns true.
__device__ __forceinline__ bool group_fold(const float *rows, float *grow, unsigned *ticket, unsigned cta,
                                           unsigned nact, bool plain) {
    constexpr unsigned S = kSubsets;
    __shared__ float wsum[S][32];
    __shared__ float lsum[S][32];
    __shared__ bool flag;
    const unsigned c = threadIdx.x & 31, sub = threadIdx.x >> 5;
    const unsigned g = cta / kGroup;
    const unsigned g0 = g * kGroup;
    const unsigned gsize = min(kGroup, nact - g0);
    if (threadIdx.x == 0) flag = (atomicAdd(&ticket[g], 1u) == gsize - 1);
    __syncthreads();
    if (!flag) return false;
    __threadfence();
    {  // subset `sub` folds rows g0 + sub + S*q
        float h = 0.0f, l = 0.0f, x[kGroup / S];
#pragma unroll
        for (unsigned q = 0; q < kGroup / S; ++q) {
            const unsigned row = sub + S * q;
            x[q] = row < gsize ? __ldcg(rows + (g0 + row) * 32 + c) : 0.0f;
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
        grow[g * 64 + 32 + c] = plain ? 0.0f : l;  // plain: the same order, no error terms
    }
    if (threadIdx.x == 0) atomicExch(&ticket[g], 0u);
    __threadfence();
    __syncthreads();
    return true;
}

// Stage 3: a group folder takes the grid ticket; the last of the `ngroups`
// folds the group rows (compensated FP32 per subset, subsets added in FP64)
// into tot[0..31] (shared), resets the ticket and returns true.
__device__ __forceinline__ bool grid_fold(const float *grow, unsigned *ticket, unsigned ngroups, double *tot,
                                          bool plain) {
    constexpr unsigned S = kSubsets;
    __shared__ double dsum[S][32];
    __shared__ bool flag;
    const unsigned c = threadIdx.x & 31, sub = threadIdx.x >> 5;
    if (threadIdx.x == 0) flag = (atomicAdd(ticket, 1u) == ngroups - 1);
    __syncthreads();
    if (!flag) return false;
    __threadfence();
    {
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
        dsum[sub][c] = plain ? (double)h : (double)h + (double)l;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        if (plain) {
            float s = 0.0f;
#pragma unroll
            for (unsigned k = 0; k < S; ++k) s += (float)dsum[k][threadIdx.x];
            tot[threadIdx.x] = (double)s;
        } else {
            double s = 0.0;
#pragma unroll
            for (unsigned k = 0; k < S; ++k) s += dsum[k][threadIdx.x];
            tot[threadIdx.x] = s;
        }
    }
    if (threadIdx.x == 0) atomicExch(ticket, 0u);
    __syncthreads();
    return true;
}

__device__ __forceinline__ bool grid_reduce32(float v[32], float *partial, float *grow, unsigned *counters,
                                              double *tot, bool plain) {
    cta_row32(v, partial + blockIdx.x * 32);
    if (!group_fold(partial, grow, counters + 1, blockIdx.x, gridDim.x, plain)) return false;
    return grid_fold(grow, counters, (gridDim.x + kGroup - 1) / kGroup, tot, plain);
}

// ---------------------------------------------------------------- estimate helpers
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
// One rounding per operation, in a fixed order, so that the pixels it sends
// inside or outside the image are the oracle's.
__device__ __forceinline__ void make_rkinv(const float *T, const LevelCam &c, float *RK) {
    const float cxi = __fmul_rn(c.cx, c.invfx), cyi = __fmul_rn(c.cy, c.invfy);
    for (int i = 0; i < 3; ++i) {
        RK[i * 3 + 0] = __fmul_rn(T[i * 4 + 0], c.invfx);
        RK[i * 3 + 1] = __fmul_rn(T[i * 4 + 1], c.invfy);
        RK[i * 3 + 2] = __fsub_rn(__fsub_rn(T[i * 4 + 2], __fmul_rn(T[i * 4 + 0], cxi)), __fmul_rn(T[i * 4 + 1], cyi));
    }
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

// The discrete decisions of the tracker (which reference pixels project
// inside the current image, which model point pairs with which current pixel
// and passes the ICP gates) and the ICP residual that GetTransform's
// keep-the-better-estimate test sums are evaluated with one IEEE rounding per
// operation in a fixed order (no contraction), exactly as the oracle
// evaluates them, so both sides take the same decisions at the same FP32
// pose.  A coordinate is tested as a float before it is converted, so a NaN
// or infinite projection is outside on both sides.

// Photometric projection of a warped reference point (se3StepRGBFunctor's
// bounds, TrackingUtils.h:73-150): inside when 0 < u < w-1 and 0 < v < h-1.
__device__ __forceinline__ bool rgb_project(const LevelCam &c, const float3 &p, float &u, float &v) {
    u = __fadd_rn(__fdiv_rn(__fmul_rn(c.fx, p.x), p.z), c.cx);
    v = __fadd_rn(__fdiv_rn(__fmul_rn(c.fy, p.y), p.z), c.cy);
    return u > 0.0f && v > 0.0f && u < (float)(c.w - 1) && v < (float)(c.h - 1);
}

__device__ __forceinline__ float dot3_rn(float a0, float a1, float a2, float b0, float b1, float b2) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)), __fmul_rn(a2, b2));
}

// IcpStepFunctor::ProjectPoint (RGBDTracking.cu:326-358) for model pixel k:
// the model point and normal moved by T, the nearest current pixel
// (floor(fx x / z + cx + 0.5)), and the gates |n_c x n_m| < sin 20 deg,
// |v_m - v_c| <= dist_th, both normals valid.  On success vl, nl, vc and the
// point-to-plane residual r = n_m . (v_c - v_m) are set.
__device__ __forceinline__ bool icp_match_vm(const float *T, const LevelCam &c, const float4 vm,
                                             const float4 *__restrict__ ref_nmap, const float4 *__restrict__ cur_vmap,
                                             const float4 *__restrict__ cur_nmap, int k, float angle_th, float dist_th,
                                             float3 &vl, float3 &nl, float4 &vc, float &r) {
    if (!(vm.w >= 0.0f)) return false;
    vl = make_float3(__fadd_rn(dot3_rn(T[0], T[1], T[2], vm.x, vm.y, vm.z), T[3]),
                     __fadd_rn(dot3_rn(T[4], T[5], T[6], vm.x, vm.y, vm.z), T[7]),
                     __fadd_rn(dot3_rn(T[8], T[9], T[10], vm.x, vm.y, vm.z), T[11]));
    const float invz = __fdiv_rn(1.0f, vl.z);
    const float fu = floorf(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(c.fx, vl.x), invz), c.cx), 0.5f));
    const float fv = floorf(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(c.fy, vl.y), invz), c.cy), 0.5f));
    if (!(fu >= 0.0f && fv >= 0.0f && fu < (float)c.w && fv < (float)c.h)) return false;
    const int q = (int)fv * c.w + (int)fu;
    vc = __ldg(cur_vmap + q);
    if (!(vc.w >= 0.0f)) return false;
    const float4 nm = __ldg(ref_nmap + k);
    nl = make_float3(dot3_rn(T[0], T[1], T[2], nm.x, nm.y, nm.z), dot3_rn(T[4], T[5], T[6], nm.x, nm.y, nm.z),
                     dot3_rn(T[8], T[9], T[10], nm.x, nm.y, nm.z));
    const float4 nc = __ldg(cur_nmap + q);
    const float dx = __fsub_rn(vl.x, vc.x), dy = __fsub_rn(vl.y, vc.y), dz = __fsub_rn(vl.z, vc.z);
    const float dist = __fsqrt_rn(dot3_rn(dx, dy, dz, dx, dy, dz));
    const float ax = __fsub_rn(__fmul_rn(nc.y, nl.z), __fmul_rn(nc.z, nl.y));
    const float ay = __fsub_rn(__fmul_rn(nc.z, nl.x), __fmul_rn(nc.x, nl.z));
    const float az = __fsub_rn(__fmul_rn(nc.x, nl.y), __fmul_rn(nc.y, nl.x));
    const float angle = __fsqrt_rn(dot3_rn(ax, ay, az, ax, ay, az));
    if (!(angle < angle_th && dist <= dist_th && nm.w > 0.0f && nc.w > 0.0f)) return false;
    r = dot3_rn(nl.x, nl.y, nl.z, __fsub_rn(vc.x, vl.x), __fsub_rn(vc.y, vl.y), __fsub_rn(vc.z, vl.z));
    return true;
}
__device__ __forceinline__ bool icp_match(const float *T, const LevelCam &c, const float4 *__restrict__ ref_vmap,
                                          const float4 *__restrict__ ref_nmap, const float4 *__restrict__ cur_vmap,
                                          const float4 *__restrict__ cur_nmap, int k, float angle_th, float dist_th,
                                          float3 &vl, float3 &nl, float4 &vc, float &r) {
    return icp_match_vm(T, c, __ldg(ref_vmap + k), ref_nmap, cur_vmap, cur_nmap, k, angle_th, dist_th, vl, nl, vc, r);
}

// The ICP row [n, v x n | r] of a matched pair, accumulated into the 28
// products (the r^2 term as the sum of rounded squares, as the oracle sums
// it) and the count.
__device__ __forceinline__ void icp_accumulate(const float3 &vl, const float3 &nl, float r, float acc[32]) {
    float row[6];
    row[0] = nl.x;
    row[1] = nl.y;
    row[2] = nl.z;
    row[3] = vl.y * nl.z - vl.z * nl.y;
    row[4] = vl.z * nl.x - vl.x * nl.z;
    row[5] = vl.x * nl.y - vl.y * nl.x;
    int q = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
#pragma unroll
        for (int j = i; j < 6; ++j) acc[q++] += row[i] * row[j];
        acc[q++] += row[i] * r;
    }
    acc[27] = __fadd_rn(acc[27], __fmul_rn(r, r));
    acc[28] += 1.0f;
}

__device__ __forceinline__ float bilinear(const float *__restrict__ m, int w, float x, float y) {
    const int u = (int)floorf(x), v = (int)floorf(y);
    const float cx = x - (float)u, cy = y - (float)v;
    const float *r0 = m + (size_t)v * w + u, *r1 = r0 + w;
    return (__ldg(r0) * (1.0f - cx) + __ldg(r0 + 1) * cx) * (1.0f - cy) +
           (__ldg(r1) * (1.0f - cx) + __ldg(r1 + 1) * cx) * cy;
}

// Huber threshold 4.685 * stddev of the photometric residuals, in FP32 as the
// reference (RGBDTracking.cu:259-278), from the double-float totals
// n = tot[29], sum r = tot[30], sum r^2 = tot[31]: mean = sum r / n, then
// sum (r - mean)^2 = sum r^2 - 2 mean sum r + n mean^2 (the reference's second
// pass over the residuals).
__device__ __forceinline__ float huber_threshold_df(DF nn, DF s, DF s2) {
    // nn.h, s.h: the totals rounded to FP32 (normalised pairs)
    const float mean = s.h / nn.h;
    const DF md = df(mean);
    const DF ss = df_fma(df_mul(nn, md), md, df_fma(df(-2.0f * mean), s, s2));
    const float var = sqrtf(ss.h / (nn.h - 1.0f));
    return (float)(4.685 * (double)var);
}
__device__ __forceinline__ float huber_threshold(const double *tot) {
    return huber_threshold_df(df_from_double(tot[29]), df_from_double(tot[30]), df_from_double(tot[31]));
}
__device__ __forceinline__ float huber_threshold_solve() {
    return huber_threshold_df(total(0, 29), total(0, 30), total(0, 31));
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
                const float z = __fdiv_rn(1.0f, zinv);
                const float3 p = warp_ref_point(sRK, sT, x, y, z);
                float u, v;
                if (rgb_project(c, p, u, v)) {
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
            float3 vl, nl;
            float4 vc;
            float r;
            if (icp_match(sT, c, a.ref_vmap, a.ref_nmap, a.cur_vmap, a.cur_nmap, k, a.angle_th, a.dist_th, vl, nl, vc,
                          r))
                icp_accumulate(vl, nl, r, acc);
        }
    }
    if (!grid_reduce32(acc, a.partial, a.grow, a.counter, tot, st->plain_sums != 0u)) return;
    if (threadIdx.x < 32) st->a_sums[threadIdx.x] = tot[threadIdx.x];
    if (threadIdx.x == 0) st->huber_th = huber_threshold(tot);
    if (a.mode == YAS_TRACK_ICP) {
        load_solve_state(st);
        if (threadIdx.x < 32) set_total_double(0, threadIdx.x, tot[threadIdx.x]);
        if (threadIdx.x == 0) g_solve.huber_th = huber_threshold(tot);
        __syncthreads();
        if (threadIdx.x < 32) {
            gn_solve(a.mode, a.no_update, a.first_of_level, a.level);
            publish_solve(st);
        }
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
    if (!grid_reduce32(acc, a.partial, a.grow, a.counter, tot, st->plain_sums != 0u)) return;
    load_solve_state(st);
    if (threadIdx.x < 32) {
        st->b_sums[threadIdx.x] = tot[threadIdx.x];
        set_total_double(1, threadIdx.x, tot[threadIdx.x]);
        set_total_double(0, threadIdx.x, __ldcg(&st->a_sums[threadIdx.x]));
    }
    if (threadIdx.x == 0) g_solve.huber_th = th;
    __syncthreads();
    if (threadIdx.x < 32) {
        gn_solve(a.mode, a.no_update, a.first_of_level, a.level);
        publish_solve(st);
    }
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
    st->huber_th = 0.0f;
    st->epoch += 1u;  // tags of the fused schedule's rows differ from every earlier launch
    st->abort_word = 0u;
    publish_estimate(st, kargs.Kd, L);
}

// ---------------------------------------------------------------- fused schedule
// One cooperative launch runs every Gauss-Newton iteration of every level
// (GetTransform's loops, RGBDTracking.cu:161-208), one CTA per SM,
// CTA c owning the pixel range [c * chunk, (c + 1) * chunk) of each level.
// Nothing is released by one CTA to the others: each CTA publishes its row
// of partial sums as tagged 64-bit words {value, tag} (tag = launch epoch and
// iteration), every CTA polls all rows until the tags match, folds them in
// the same fixed order and runs the same solve, so every CTA holds the same
// estimate without a barrier, a fence or an atomic:
//   1. pass A (warp, photometric residual, ICP products) -> row A;
//      [RGB] fold of the three photometric moments -> Huber threshold;
//   2. [RGB] pass B (weighted photometric products, from the residuals each
//      thread kept in registers) -> row B;
//   3. fold of the ICP and photometric systems -> solve -> estimate.
// Rows are double-buffered by iteration parity: a CTA can run at most one
// iteration ahead of the slowest reader of a buffer.  Every wait is bounded by
// a wall-clock limit: a CTA that gives up raises the state's abort word, every
// waiter leaves as soon as it sees it, and the state reports kFailTimeout.
// CTA 0 writes the final state to global memory.
// CTA size NT: 512 threads when every thread keeps its pixels' residuals in
// registers (PIX = 1, 2, 4), 1024 otherwise (PIX = 0, and the batched
// schedules, whose CTAs own many pixels each and are latency-bound on them).
// A row costs each warp a 31-shuffle transpose reduction (shuffles issue at
// one warp instruction per cycle per SM), so 512 threads halve that
// twice-per-iteration cost, and 128 registers per thread hold four level-0
// pixels' residuals without spills (measured at 640x480: 244 against 252 us
// per launch; the batched and the PIX = 0 schedules were slower at 512).
constexpr int kFusedMaxCtas = 160;  // rows the system fold covers
template <int PIX>
constexpr int fused_threads() { return PIX == 0 ? 1024 : 512; }
constexpr int kBatchThreads = 1024;
template <int NT>
struct FoldShape {
    static constexpr int warps = NT / 32;
    static constexpr int subsets = NT / 64;                 // row subsets of the system fold
    static constexpr int rows = kFusedMaxCtas / subsets;    // rows per subset
    static_assert(subsets * rows == kFusedMaxCtas && 3 * kFusedMaxCtas <= NT, "fold shape");
};
constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s


struct FusedArgs {
    FusedLevel lv[kMaxLevels];
    int L, mode;
    float angle_th, dist_th;
    unsigned long long *rows;  // [2 parities][2 passes][kFusedMaxCtas][32] tagged words
    float4 *res4;              // per-pixel residuals of the PIX == 0 schedule (level-0 sized)
    GNState *st;
};

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long tagged(float x, unsigned tag) {
    return ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(x);
}

__device__ __forceinline__ bool tag_is(unsigned long long w, unsigned tag) { return (unsigned)(w >> 32) == tag; }

// One step of a bounded poll: false once the launch was aborted or this
// thread's wait (started at t0) exceeded kWaitLimitNs, which it then reports.
__device__ __forceinline__ bool poll_continue(GNState *st, unsigned spin, unsigned long long &t0) {
    __nanosleep(spin < 32 ? 32 : 256);
    if ((spin & 15u) != 15u) return true;
    if (ld_relaxed_u32(&st->abort_word) != 0u) return false;
    const unsigned long long now = global_ns();
    if (t0 == 0ull) {
        t0 = now;
    } else if (now - t0 > kWaitLimitNs) {
        st->failed = kFailTimeout;
        atomicExch(&st->abort_word, 1u);
        return false;
    }
    return true;
}

// Pass A for one pixel whose reference depth (1 / inverse depth, 0 where
// that is invalid: the same division gn_pass_a makes) and model vertex are
// already loaded: the photometric residual (kept in registers for pass B)
// and the ICP products, accumulated as gn_pass_a does.
__device__ __forceinline__ void fused_pixel_a_pre(const FusedLevel &lv, const float *sT, const float *sRK, int k,
                                                  bool do_rgb, bool do_icp, float angle_th, float dist_th,
                                                  float z, float4 vm, float acc[32], float4 &res, float3 &p) {
    const LevelCam &c = lv.c;
    const int y = k / c.w, x = k - y * c.w;
    res = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    p = make_float3(0.0f, 0.0f, 1.0f);
    if (do_rgb) {
        if (z > 0.0f) {
            p = warp_ref_point(sRK, sT, x, y, z);
            float u, v;
            if (rgb_project(c, p, u, v)) {
                const float r = bilinear(lv.cur_int, c.w, u, v) - __ldg(lv.ref_int + k);
                const float gx = bilinear(lv.cur_gx, c.w, u, v);
                const float gy = bilinear(lv.cur_gy, c.w, u, v);
                const bool ok = (gx * gx + gy * gy) > 0.0f && isfinite(r);
                res = make_float4(r, gx, gy, ok ? 1.0f : -1.0f);
                if (ok) {
                    acc[29] += 1.0f;
                    acc[30] += r;
                    acc[31] += r * r;
                }
            }
        }
    }
    if (do_icp) {
        float3 vl, nl;
        float4 vc;
        float r;
        if (icp_match_vm(sT, c, vm, lv.ref_nmap, lv.cur_vmap, lv.cur_nmap, k, angle_th, dist_th, vl, nl, vc, r))
            icp_accumulate(vl, nl, r, acc);
    }
}

// Pass A for one pixel: the photometric residual (kept in registers for pass
// B) and the ICP products, accumulated as gn_pass_a does.
__device__ __forceinline__ void fused_pixel_a(const FusedLevel &lv, const float *sT, const float *sRK, int k,
                                              bool do_rgb, bool do_icp, float angle_th, float dist_th,
                                              float acc[32], float4 &res, float3 &p) {
    fused_pixel_a_pre(lv, sT, sRK, k, do_rgb, do_icp, angle_th, dist_th, do_rgb ? __ldg(lv.ref_z + k) : 0.0f,
                      do_icp ? __ldg(lv.ref_vmap + k) : make_float4(0.0f, 0.0f, 0.0f, -1.0f), acc, res, p);
}

// Pass B for one pixel kept from pass A (gn_pass_b's products).
__device__ __forceinline__ void fused_pixel_b(const LevelCam &c, float th, const float4 &res, const float3 &p,
                                              float acc[32]) {
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


// The CTA's row of 32 sums (warp transpose sums, then a pairwise tree over
// the 32 warp sums of each value), published by warp 0 as tagged words.
template <int NT>
__device__ __forceinline__ void fused_publish_row(float v[32], unsigned long long *row, unsigned tag) {
    constexpr int kFusedWarps = FoldShape<NT>::warps;
    __shared__ float wsum[kFusedWarps][33];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const float r = warp_transpose_reduce(v);
    wsum[warp][lane] = r;
    __syncthreads();
    if (warp == 0) {
        float x[kFusedWarps];
#pragma unroll
        for (int w = 0; w < kFusedWarps; ++w) x[w] = wsum[w][lane];
#pragma unroll
        for (int s = kFusedWarps / 2; s >= 1; s >>= 1)
#pragma unroll
            for (int i = 0; i < s; ++i) x[i] += x[i + s];
        st_relaxed_u64(row + lane, tagged(x[0], tag));
    }
}

// Totals over all CTAs of the photometric moments (columns 29..31 of rows A)
// into the solve's totals 29..31 of pass A; compensated FP32 per column (32
// lanes x 5 rows, then a butterfly), kept as a double-float pair.  False on
// abort or timeout.
__device__ __forceinline__ bool fold_moments(const unsigned long long *rows, unsigned nrows, unsigned tag,
                                             GNState *st, bool plain) {
    __shared__ float m3[3][kFusedMaxCtas];
    const int t = (int)threadIdx.x;
    bool mine = true;
    if (t < 3 * (int)nrows) {
        const int q = t / (int)nrows, r = t - q * (int)nrows;
        const unsigned long long *p = rows + r * 32 + 29 + q;
        unsigned long long w = ld_relaxed_u64(p);
        unsigned long long t0 = 0ull;
        for (unsigned spin = 0; !tag_is(w, tag); ++spin) {
            if (!poll_continue(st, spin, t0)) {
                mine = false;
                break;
            }
            w = ld_relaxed_u64(p);
        }
        m3[q][r] = __uint_as_float((unsigned)w);
    }
    if (!__syncthreads_and(mine)) return false;
    const int warp = t >> 5, lane = t & 31;
    if (warp < 3) {
        float h = 0.0f, l = 0.0f;
#pragma unroll
        for (int m = 0; m < (kFusedMaxCtas + 31) / 32; ++m) {
            const int r = lane + 32 * m;
            float s, e;
            two_sum(h, r < (int)nrows ? m3[warp][r] : 0.0f, s, e);
            h = s;
            l += e;
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, h, off), ol = __shfl_xor_sync(0xffffffffu, l, off);
            float s, e;
            two_sum(h, oh, s, e);
            h = s;
            l = (l + ol) + e;
        }
        if (lane == 0) set_total(0, 29 + warp, h, plain ? 0.0f : l);
    }
    __syncthreads();
    return true;
}

// Totals over all CTAs of the ICP system (columns 0..28 of rows A) into the
// solve's pass A totals 0..28 and of the photometric system (columns 0..27 of
// rows B) into its pass B totals 0..27 (zero for a term the mode does not
// use).  Thread t folds column t % 64 over the rows of subset t / 64
// (compensated FP32), then a butterfly over the subsets of each column (8 at
// 512 threads, 16 at 1024);
// each total is kept as a double-float pair.  False on abort or timeout.
template <int NT>
__device__ __forceinline__ bool fold_systems(const unsigned long long *rowsA, const unsigned long long *rowsB,
                                             unsigned nrows, unsigned tag, bool icp, bool rgb, GNState *st,
                                             bool plain) {
    constexpr int kFoldSubsets = FoldShape<NT>::subsets, kFoldRows = FoldShape<NT>::rows;
    constexpr int kFusedWarps = FoldShape<NT>::warps;
    __shared__ float hs[kFoldSubsets][65], ls[kFoldSubsets][65];
    const int t = (int)threadIdx.x, c = t & 63, sub = t >> 6;
    const bool need = (c < 29 && icp) || (c >= 32 && c < 60 && rgb);
    bool mine = true;
    float h = 0.0f, l = 0.0f;
    if (need) {
        const unsigned long long *base = c < 32 ? rowsA + c : rowsB + (c - 32);
        unsigned long long w[kFoldRows];
#pragma unroll
        for (int q = 0; q < kFoldRows; ++q) {
            const unsigned r = (unsigned)(sub + kFoldSubsets * q);
            w[q] = r < nrows ? ld_relaxed_u64(base + r * 32) : tagged(0.0f, tag);
        }
        unsigned long long t0 = 0ull;
        for (unsigned spin = 0;; ++spin) {
            unsigned pend = 0u;
#pragma unroll
            for (int q = 0; q < kFoldRows; ++q)
                if (!tag_is(w[q], tag)) pend |= 1u << q;
            if (pend == 0u) break;
            if (!poll_continue(st, spin, t0)) {
                mine = false;
                break;
            }
#pragma unroll
            for (int q = 0; q < kFoldRows; ++q)
                if ((pend >> q) & 1u) w[q] = ld_relaxed_u64(base + (sub + kFoldSubsets * q) * 32);
        }
#pragma unroll
        for (int q = 0; q < kFoldRows; ++q) {
            float s, e;
            two_sum(h, __uint_as_float((unsigned)w[q]), s, e);
            h = s;
            l += e;
        }
    }
    hs[sub][c] = h;
    ls[sub][c] = l;
    if (!__syncthreads_and(mine)) return false;
    {  // warp w folds columns n w + c (n = 64 / warps), lanes c S .. c S + S - 1 = the S subsets
        constexpr int kColsPerWarp = 64 / kFusedWarps;
        const int warp = t >> 5, lane = t & 31;
        const int col = kColsPerWarp * warp + lane / kFoldSubsets, s_ = lane % kFoldSubsets;
        float h2 = hs[s_][col], l2 = ls[s_][col];
#pragma unroll
        for (int off = kFoldSubsets / 2; off >= 1; off >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, h2, off), ol = __shfl_xor_sync(0xffffffffu, l2, off);
            float s, e;
            two_sum(h2, oh, s, e);
            h2 = s;
            l2 = (l2 + ol) + e;
        }
        if (s_ == 0) {
            if (col < 29) set_total(0, col, h2, plain ? 0.0f : l2);
            else if (col >= 32 && col < 60) set_total(1, col - 32, h2, plain ? 0.0f : l2);
        }
    }
    __syncthreads();
    return true;
}

// The fused schedule of one tracker, run by `nrows` CTAs (this one is `cta`).
// Level l's pixel k = cta * chunk_l + off, off < chunk_l.  PIX > 0: a thread
// owns at most PIX pixels per level (off = s * NT + thread, NT threads) and
// keeps their residuals in registers for pass B; PIX == 0: any number of
// pixels, residuals through `res4` (pass B then recomputes the warped point,
// as gn_pass_b does), G pixels' reference loads at a time.
template <int PIX, int NT, int G>
__device__ __forceinline__ void gn_schedule(const FusedLevel *lvs, int L, int mode, float angle_th, float dist_th,
                                            unsigned long long *rows, float4 *res4, GNState *st, unsigned cta,
                                            unsigned nrows) {
    __shared__ float sRK[9];
    const int t = (int)threadIdx.x;
    const bool do_rgb = (mode & YAS_TRACK_RGB) != 0, do_icp = (mode & YAS_TRACK_ICP) != 0;
    load_solve_state(st);
    if (t >= 32 && t < 64) {
        g_solve.Ah[t - 32] = 0.0f;
        g_solve.Al[t - 32] = 0.0f;
        g_solve.Bh[t - 32] = 0.0f;
        g_solve.Bl[t - 32] = 0.0f;
    }
    const unsigned epoch = __ldcg(&st->epoch);
    const bool plain = __ldcg(&st->plain_sums) != 0u;
    __syncthreads();
    unsigned s = 0u;
    bool alive = true;
    for (int l = L - 1; l >= 0 && alive; --l) {
        const FusedLevel &lv = lvs[l];
        const int n = lv.c.w * lv.c.h;
        const int base = (int)cta * lv.chunk;
        for (int it = 0; it < lv.iters; ++it) {
            ++s;
            const unsigned tag = (epoch << 12) | (s & 0xfffu);
            unsigned long long *rA = rows + (size_t)((s & 1u) * 2u + 0u) * kFusedMaxCtas * 32;
            unsigned long long *rB = rows + (size_t)((s & 1u) * 2u + 1u) * kFusedMaxCtas * 32;
            if (t == 0) make_rkinv(g_solve.Tf, lv.c, sRK);
            __syncthreads();
            float acc[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) acc[i] = 0.0f;
            float4 res[PIX > 0 ? PIX : 1];
            float3 pp[PIX > 0 ? PIX : 1];
            if constexpr (PIX > 0) {
                // the pose-independent reference loads (depth, model vertex) of
                // every pixel first, so they are in flight together
                float zi[PIX];
                float4 vm[PIX];
#pragma unroll
                for (int q = 0; q < PIX; ++q) {
                    const int off = q * NT + t;
                    const int k = base + off;
                    const bool own = q < lv.pix && off < lv.chunk && k < n;
                    zi[q] = own && do_rgb ? __ldg(lv.ref_z + k) : 0.0f;
                    vm[q] = own && do_icp ? __ldg(lv.ref_vmap + k) : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
                }
#pragma unroll
                for (int q = 0; q < PIX; ++q) {
                    res[q] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
                    pp[q] = make_float3(0.0f, 0.0f, 1.0f);
                    const int off = q * NT + t;
                    const int k = base + off;
                    if (q < lv.pix && off < lv.chunk && k < n)
                        fused_pixel_a_pre(lv, g_solve.Tf, sRK, k, do_rgb, do_icp, angle_th, dist_th, zi[q], vm[q], acc,
                                          res[q], pp[q]);
                }
            } else {
                // pixels off = t, t + NT, ... in groups of G, each group's
                // reference loads first (the same pixels in the same order as
                // one at a time); G = 2 in the batched schedules, whose CTAs
                // own tens of pixels per thread, G = 1 where a second
                // pixel's registers would spill (1024 threads, 64 registers)
#pragma unroll 1
                for (int off0 = t; off0 < lv.chunk; off0 += G * NT) {
                    float zi[G];
                    float4 vm[G];
#pragma unroll
                    for (int q = 0; q < G; ++q) {
                        const int off = off0 + q * NT, k = base + off;
                        const bool own = off < lv.chunk && k < n;
                        zi[q] = own && do_rgb ? __ldg(lv.ref_z + k) : 0.0f;
                        vm[q] = own && do_icp ? __ldg(lv.ref_vmap + k) : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
                    }
#pragma unroll
                    for (int q = 0; q < G; ++q) {
                        const int off = off0 + q * NT, k = base + off;
                        if (off >= lv.chunk || k >= n) break;
                        float4 r4;
                        float3 p3;
                        fused_pixel_a_pre(lv, g_solve.Tf, sRK, k, do_rgb, do_icp, angle_th, dist_th, zi[q], vm[q], acc,
                                          r4, p3);
                        if (do_rgb) res4[k] = r4;
                    }
                }
            }
            fused_publish_row<NT>(acc, rA + cta * 32, tag);
            if (do_rgb) {
                if (!fold_moments(rA, nrows, tag, st, plain)) return;
                if (t == 0) g_solve.huber_th = huber_threshold_solve();
                __syncthreads();
                const float th = g_solve.huber_th;
#pragma unroll
                for (int i = 0; i < 32; ++i) acc[i] = 0.0f;
                if constexpr (PIX > 0) {
#pragma unroll
                    for (int q = 0; q < PIX; ++q)
                        if (res[q].w > 0.0f) fused_pixel_b(lv.c, th, res[q], pp[q], acc);
                } else {
#pragma unroll 1
                    for (int off0 = t; off0 < lv.chunk; off0 += G * NT) {
                        float4 r4[G];
                        float zi[G];
#pragma unroll
                        for (int q = 0; q < G; ++q) {
                            const int off = off0 + q * NT, k = base + off;
                            const bool own = off < lv.chunk && k < n;
                            r4[q] = own ? res4[k] : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
                            zi[q] = own ? __ldg(lv.ref_z + k) : 1.0f;
                        }
#pragma unroll
                        for (int q = 0; q < G; ++q) {
                            const int k = base + off0 + q * NT;
                            if (r4[q].w > 0.0f) {
                                const int y = k / lv.c.w, x = k - y * lv.c.w;
                                const float3 p3 = warp_ref_point(sRK, g_solve.Tf, x, y, zi[q]);
                                fused_pixel_b(lv.c, th, r4[q], p3, acc);
                            }
                        }
                    }
                }
                fused_publish_row<NT>(acc, rB + cta * 32, tag);
            }
            if (!fold_systems<NT>(rA, rB, nrows, tag, do_icp, do_rgb, st, plain)) return;
            if (t < 32) {
                if (!do_rgb && t == 0) g_solve.huber_th = huber_threshold_solve();
                if constexpr (NT <= 512)
                    gn_solve_inline(mode, 0, it == 0, l);
                else
                    gn_solve(mode, 0, it == 0, l);
            }
            __syncthreads();
            if (g_solve.failed != 0) {
                alive = false;
                break;
            }
        }
    }
    if (cta == 0 && t < 32) {
        publish_solve(st);
        st->a_sums[t] = df_to_double(total(0, t));
        st->b_sums[t] = df_to_double(total(1, t));
    }
}

// The fused schedule of one tracker over the whole grid.
template <int PIX>
__global__ void __launch_bounds__(fused_threads<PIX>(), 1) gn_fused(const __grid_constant__ FusedArgs a) {
    gn_schedule<PIX, fused_threads<PIX>(), 1>(a.lv, a.L, a.mode, a.angle_th, a.dist_th, a.rows, a.res4, a.st, blockIdx.x, gridDim.x);
}

// Fused schedules of a batch of trackers in one launch: CTA b runs for item
// cta_item[b] as its CTA b - cta0 of nctas.  Items never wait on each other,
// so an item's result is the same alone and in any batch.
// PIX > 0: every item's CTAs own at most PIX pixels per thread on every level
// (residuals kept in registers); PIX == 0: any share (residuals in res4).
template <int PIX>
__global__ void __launch_bounds__(kBatchThreads, 1) gn_fused_batch(const GNBatchItem *__restrict__ items,
                                                                    const unsigned short *__restrict__ cta_item) {
    const GNBatchItem &it = items[cta_item[blockIdx.x]];
    gn_schedule<PIX, kBatchThreads, 2>(it.lv, it.L, it.mode, it.angle_th, it.dist_th, it.rows, it.res4, it.st,
                                    blockIdx.x - (unsigned)it.cta0, (unsigned)it.nctas);
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


template <int PIX>
static cudaError_t launch_fused_pix(const FusedArgs &a, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(fused_threads<PIX>());
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, gn_fused<PIX>, a);
}

// Grid of the fused schedule: one CTA per SM (512 threads; 1024 for PIX = 0),
// at most kFusedMaxCtas (the rows the system fold covers).  Level l gives each CTA a
// chunk of ceil(P_l / grid) pixels rounded up to a warp; `pix` is the smallest
// compiled pixels-per-thread bound (1, 2 or 4) that covers level 0's chunk,
// or 0 (any chunk, residuals through global memory) when none does.  Returns
// false without cooperative launch (the per-iteration launches are used).
static bool fused_plan(yas_tracker *tr, int &pix, int &grid) {
    if (tr->fused_max_grid[0] < 0) {
        int dev = 0, sms = 0, coop = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        int nb[4] = {0, 0, 0, 0};
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[0], gn_fused<1>, fused_threads<1>(), 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[1], gn_fused<2>, fused_threads<2>(), 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[2], gn_fused<4>, fused_threads<4>(), 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[3], gn_fused<0>, fused_threads<0>(), 0);
        cudaGetLastError();
        // one CTA per SM (the schedule's design), whatever else would fit
        for (int i = 0; i < 4; ++i)
            tr->fused_max_grid[i] = coop ? std::min(std::min(nb[i], 1) * sms, kFusedMaxCtas) : 0;
    }
    const long long P0 = (long long)tr->cam[0].w * tr->cam[0].h;
    const int pixes[3] = {1, 2, 4};
    for (int i = 0; i < 3; ++i) {
        const int g = tr->fused_max_grid[i];
        if (g <= 0) continue;
        const long long chunk = ((P0 + g - 1) / g + 31) / 32 * 32;
        if (chunk <= (long long)fused_threads<1>() * pixes[i]) {
            pix = pixes[i];
            grid = g;
            return true;
        }
    }
    // larger frames (e.g. 1280x720 on 152 SMs): residuals through global memory
    if (tr->fused_max_grid[3] > 0) {
        pix = 0;
        grid = tr->fused_max_grid[3];
        return true;
    }
    return false;
}

// Levels of a fused schedule run by `grid` CTAs, on the tracker's current sets.
static void fill_levels(yas_tracker *tr, int grid, int threads, FusedLevel *lv) {
    for (int l = 0; l < tr->L; ++l) {
        FusedLevel &f = lv[l];
        f.c = tr->cam[l];
        f.iters = tr->iters[l];
        const long long P = (long long)f.c.w * f.c.h;
        f.chunk = (int)(((P + grid - 1) / grid + 31) / 32 * 32);
        f.pix = (f.chunk + threads - 1) / threads;
        TrackLevelBufs &cb = tr->curb(l), &rb = tr->refb(l);
        f.ref_int = rb.intensity;
        f.ref_invd = rb.invd;
        f.ref_z = rb.z;
        f.ref_vmap = rb.vmap;
        f.ref_nmap = rb.nmap;
        f.cur_int = cb.intensity;
        f.cur_gx = tr->gx[l];
        f.cur_gy = tr->gy[l];
        f.cur_vmap = cb.vmap;
        f.cur_nmap = cb.nmap;
    }
}

static bool launch_gn_fused(yas_tracker *tr, cudaStream_t s) {
    int pix = 0, grid = 0;
    if (!tr->use_fused || !fused_plan(tr, pix, grid)) return false;
    FusedArgs a;
    memset(&a, 0, sizeof(a));
    fill_levels(tr, grid, pix == 0 ? fused_threads<0>() : fused_threads<1>(), a.lv);
    a.L = tr->L;
    a.mode = tr->mode;
    a.angle_th = tr->angle_th;
    a.dist_th = tr->dist_th;
    a.rows = tr->fused_rows;
    a.res4 = tr->res4;
    a.st = tr->state;
    if (tr->hook) tr->hook(tr->hook_ctx, 30);
    const cudaError_t e = pix == 1   ? launch_fused_pix<1>(a, grid, s)
                          : pix == 2 ? launch_fused_pix<2>(a, grid, s)
                          : pix == 4 ? launch_fused_pix<4>(a, grid, s)
                                     : launch_fused_pix<0>(a, grid, s);
    if (e != cudaSuccess) {
        // e.g. a device without cooperative launch: use the per-iteration launches
        cudaGetLastError();
        tr->use_fused = false;
        return false;
    }
    return true;
}

// A tracker takes a fixed number of CTAs in a batch, set by its resolution
// alone (one per 32 Ki level-0 pixels, 1..16), so its result does not depend
// on the rest of the batch.
int gn_batch_ctas(const yas_tracker *tr, int pixels_per_cta) {
    const long long P0 = (long long)tr->cam[0].w * tr->cam[0].h;
    const long long q = std::max(1024, pixels_per_cta);
    return (int)std::min<long long>(16, std::max<long long>(1, (P0 + q - 1) / q));
}

void gn_batch_item(yas_tracker *tr, int cta0, GNBatchItem *out, int pixels_per_cta) {
    gn_batch_item_ctas(tr, cta0, gn_batch_ctas(tr, pixels_per_cta), out);
}

void gn_batch_item_ctas(yas_tracker *tr, int cta0, int nctas, GNBatchItem *out) {
    memset(out, 0, sizeof(*out));
    out->nctas = std::max(1, std::min(nctas, kFusedMaxCtas));
    out->cta0 = cta0;
    fill_levels(tr, out->nctas, kBatchThreads, out->lv);
    out->L = tr->L;
    out->mode = tr->mode;
    out->angle_th = tr->angle_th;
    out->dist_th = tr->dist_th;
    out->rows = tr->fused_rows;
    out->res4 = tr->res4;
    out->st = tr->state;
}

int gn_batch_capacity() {
    static int cap[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 0;
    if (cap[dev] == 0) {
        int sms = 0, nb = 0, coop = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        int lowest = 1 << 30;
        for (auto k : {gn_fused_batch<0>, gn_fused_batch<1>, gn_fused_batch<2>, gn_fused_batch<4>}) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kBatchThreads, 0);
            lowest = std::min(lowest, nb);
        }
        cudaGetLastError();
        cap[dev] = coop ? std::max(0, std::min(std::min(lowest, 1) * sms, kFusedMaxCtas)) : -1;
    }
    return cap[dev];
}

int gn_batch_pix(const GNBatchItem *items, int n) {
    int pix = 0;
    for (int i = 0; i < n; ++i)
        for (int l = 0; l < items[i].L; ++l) pix = std::max(pix, items[i].lv[l].pix);
    return pix <= 1 ? 1 : (pix <= 2 ? 2 : (pix <= 4 ? 4 : 0));
}

cudaError_t launch_gn_batch(const GNBatchItem *dev_items, const unsigned short *dev_cta_item, int grid,
                            cudaStream_t s, int pix) {
    if (grid <= 0 || grid > gn_batch_capacity()) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBatchThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    switch (pix) {
        case 1: return cudaLaunchKernelEx(&cfg, gn_fused_batch<1>, dev_items, dev_cta_item);
        case 2: return cudaLaunchKernelEx(&cfg, gn_fused_batch<2>, dev_items, dev_cta_item);
        case 4: return cudaLaunchKernelEx(&cfg, gn_fused_batch<4>, dev_items, dev_cta_item);
        default: return cudaLaunchKernelEx(&cfg, gn_fused_batch<0>, dev_items, dev_cta_item);
    }
}

void launch_gn_schedule(yas_tracker *tr, cudaStream_t s) {
    if (launch_gn_fused(tr, s)) return;
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
            b.z = (float *)grab(n * 4);
            b.vmap = (float4 *)grab(n * 16);
            b.nmap = (float4 *)grab(n * 16);
            if (!b.intensity || !b.invd || !b.z || !b.vmap || !b.nmap) return YAS_ERR_OOM;
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
    tr->fused_rows = (unsigned long long *)grab((size_t)4 * kFusedMaxCtas * 32 * sizeof(unsigned long long));
    tr->state = (GNState *)grab(sizeof(GNState));
    tr->staging_bytes = (size_t)tr->w * tr->h * 4;
    tr->staging = grab(tr->staging_bytes);
    if (!tr->res4 || !tr->partialA || !tr->partialB || !tr->growA || !tr->growB || !tr->counters || !tr->fused_rows || !tr->state || !tr->staging)
        return YAS_ERR_OOM;
    if (cudaMallocHost(&tr->state_host, sizeof(GNState)) != cudaSuccess) {
        cudaGetLastError();
        return YAS_ERR_OOM;
    }
    memset(tr->state_host, 0, sizeof(GNState));
    // the zero fills ran on the legacy stream, which the tracker's
    // non-blocking streams do not wait for
    if (cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess) return YAS_ERR_CUDA;
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
    launch_depth_level0(src, is_u16, pitch, scale, tr->cam[0], depth_m, B[0].invd, B[0].z, B[0].vmap, B[0].nmap,
                        s);
    for (int l = 1; l < tr->L; ++l)
        launch_depth_level(B[l - 1].invd, tr->cam[l - 1].w, tr->cam[l], B[l].invd, B[l].z, B[l].vmap, B[l].nmap,
                           s);
}

void tracker_model(yas_tracker *tr, cudaStream_t s) {
    TrackLevelBufs *B = tr->set[1 - tr->cur];
    int w[kMaxLevels], h[kMaxLevels];
    float4 *vm[kMaxLevels], *nm[kMaxLevels];
    for (int l = 0; l < tr->L; ++l) {
        w[l] = tr->cam[l].w;
        h[l] = tr->cam[l].h;
        vm[l] = B[l].vmap;
        nm[l] = B[l].nmap;
    }
    launch_model_pyramid(tr->L, w, h, vm, nm, s);
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

// Device address of g_static_scratch, resolved once per device and CUDA
// context.  The module (and with it the array) is loaded again in a new
// context, e.g. after cudaDeviceReset, so the cached address is keyed on the
// context's unique id and resolved again when the current context changes.
typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);

struct StaticSlot {
    unsigned long long ctx_id;
    StaticScratch *ptr;
};
static std::mutex g_static_mutex;
static StaticSlot g_static_slot[64];
static PfnCtxGetCurrent g_ctx_get_current = nullptr;
static PfnCtxGetId g_ctx_get_id = nullptr;

// Id of the calling thread's current context (0 when there is none yet).
// Caller holds g_static_mutex.
static int current_context_id(unsigned long long *id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void *p = nullptr, *q = nullptr;
        cudaDriverEntryPointQueryResult r1 = cudaDriverEntryPointSymbolNotFound, r2 = r1;
        YAS_TRY_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &r1));
        YAS_TRY_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault, &r2));
        if (r1 != cudaDriverEntryPointSuccess || r2 != cudaDriverEntryPointSuccess || !p || !q) return YAS_ERR_STATE;
        g_ctx_get_current = reinterpret_cast<PfnCtxGetCurrent>(p);
        g_ctx_get_id = reinterpret_cast<PfnCtxGetId>(q);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return YAS_ERR_STATE;
    *id = 0;
    if (ctx && g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return YAS_ERR_STATE;
    return YAS_OK;
}

static int static_scratch(StaticScratch **out) {
    int dev = 0;
    YAS_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return YAS_ERR_STATE;
    std::lock_guard<std::mutex> lk(g_static_mutex);
    unsigned long long id = 0;
    YAS_TRY(current_context_id(&id));
    StaticSlot &slot = g_static_slot[dev];
    if (!slot.ptr || id == 0 || slot.ctx_id != id) {
        // cudaGetSymbolAddress also makes the device's primary context current
        // when no context is yet, so the id is read again afterwards
        void *p = nullptr;
        YAS_TRY_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
        YAS_TRY(current_context_id(&id));
        if (id == 0) return YAS_ERR_STATE;
        slot.ptr = static_cast<StaticScratch *>(p);
        slot.ctx_id = id;
    }
    *out = slot.ptr;
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
    LevelCam cam;
    memset(&cam, 0, sizeof(cam));
    cam.w = lv->width;
    cam.h = lv->height;
    // the pass grid must fit the static partial-sum rows and tickets
    const int g = pass_grid(cam);
    if (g > kStaticMaxCtas) return YAS_ERR_CAPACITY;
    StaticScratch *sc = nullptr;
    YAS_TRY(static_scratch(&sc));
    cudaStream_t s = (cudaStream_t)stream;
    // tickets must start at zero; everything else is written before it is read
    YAS_TRY_CUDA(cudaMemsetAsync(sc->counters, 0, sizeof(sc->counters), s));
    // compensated sums, whatever an earlier call left
    YAS_TRY_CUDA(cudaMemsetAsync(&sc->state.plain_sums, 0, sizeof(unsigned), s));
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

// ---------------------------------------------------------------- self-check of the solve's division
namespace yas {
__global__ void df_div_kernel(const double *a, const double *x, double *out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = df_to_double(df_div(df_from_double(a[i]), df_from_double(x[i])));
}
}  // namespace yas

extern "C" YAS_API int yas_check_div_seeded(const double *a, const double *x, double *out, int n) {
    using namespace yas;
    if (!a || !x || !out || n <= 0 || n > (1 << 20)) return YAS_ERR_BAD_ARG;
    const size_t bytes = sizeof(double) * (size_t)n;
    double *d = nullptr;
    YAS_TRY_CUDA(cudaMalloc(&d, 3 * bytes));
    cudaError_t e = cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, x, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        df_div_kernel<<<(n + 255) / 256, 256>>>(d, d + n, d + 2 * (size_t)n, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? YAS_OK : YAS_ERR_CUDA;
}
