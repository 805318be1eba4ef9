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
    double *partial;
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

// CTA reduction of 32 values + last-CTA FP64 combine.  Returns true in the last
// CTA, where tot[0..31] (shared) holds the grid totals.
__device__ __forceinline__ bool grid_reduce32(float v[32], double *partial, unsigned *counter,
                                              double *tot) {
    __shared__ float wsum[kTrackThreads / 32][32];
    __shared__ double gsum[kTrackThreads / 32][32];
    __shared__ bool last;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    float r = warp_transpose_reduce(v);
    wsum[warp][lane] = r;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = 0.0f;
#pragma unroll
        for (int w = 0; w < kTrackThreads / 32; ++w) s += wsum[w][threadIdx.x];
        partial[blockIdx.x * 32 + threadIdx.x] = (double)s;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned ticket = atomicAdd(counter, 1u);
        last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    {
        const unsigned c = threadIdx.x & 31, g = threadIdx.x >> 5;
        double acc = 0.0;
        for (unsigned b = g; b < gridDim.x; b += kTrackThreads / 32) acc += __ldcg(partial + b * 32 + c);
        gsum[g][c] = acc;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = 0.0;
#pragma unroll
        for (int g = 0; g < kTrackThreads / 32; ++g) s += gsum[g][threadIdx.x];
        tot[threadIdx.x] = s;
    }
    if (threadIdx.x == 0) *counter = 0u;
    __syncthreads();
    return true;
}

// ---------------------------------------------------------------- FP64 algebra
// LDL^T with diagonal pivoting (largest remaining diagonal, left-looking) and
// a pseudo-inverse of D (|d| <= 1/DBL_MAX -> 0): the algorithm of Eigen 3's LDLT.
__device__ void ldlt_solve6(const double *Ain, const double *bin, double *x) {
    double A[36];
    int tr[6];
    for (int i = 0; i < 36; ++i) A[i] = Ain[i];
    for (int k = 0; k < 6; ++k) {
        int p = k;
        double best = fabs(A[k * 6 + k]);
        for (int i = k + 1; i < 6; ++i)
            if (fabs(A[i * 6 + i]) > best) {
                best = fabs(A[i * 6 + i]);
                p = i;
            }
        tr[k] = p;
        if (p != k) {
            for (int j = 0; j < 6; ++j) {
                double t = A[k * 6 + j];
                A[k * 6 + j] = A[p * 6 + j];
                A[p * 6 + j] = t;
            }
            for (int i = 0; i < 6; ++i) {
                double t = A[i * 6 + k];
                A[i * 6 + k] = A[i * 6 + p];
                A[i * 6 + p] = t;
            }
        }
        double temp[6];
        if (k > 0) {
            for (int j = 0; j < k; ++j) temp[j] = A[j * 6 + j] * A[k * 6 + j];
            double s = 0.0;
            for (int j = 0; j < k; ++j) s += A[k * 6 + j] * temp[j];
            A[k * 6 + k] -= s;
            for (int i = k + 1; i < 6; ++i) {
                double t = 0.0;
                for (int j = 0; j < k; ++j) t += A[i * 6 + j] * temp[j];
                A[i * 6 + k] -= t;
            }
        }
        const double d = A[k * 6 + k];
        const bool valid = fabs(d) > 0.0;
        if (k == 0 && !valid) {
            // whole diagonal zero (or NaN): identity transpositions, solve as is
            for (int j = 0; j < 6; ++j) tr[j] = j;
            break;
        }
        if (valid)
            for (int i = k + 1; i < 6; ++i) A[i * 6 + k] /= d;
    }
    double y[6];
    for (int i = 0; i < 6; ++i) y[i] = bin[i];
    for (int k = 0; k < 6; ++k) {
        double t = y[k];
        y[k] = y[tr[k]];
        y[tr[k]] = t;
    }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < i; ++j) y[i] -= A[i * 6 + j] * y[j];
    const double tol = 1.0 / DBL_MAX;
    for (int i = 0; i < 6; ++i) y[i] = fabs(A[i * 6 + i]) > tol ? y[i] / A[i * 6 + i] : 0.0;
    for (int i = 5; i >= 0; --i)
        for (int j = i + 1; j < 6; ++j) y[i] -= A[j * 6 + i] * y[j];
    for (int k = 5; k >= 0; --k) {
        double t = y[k];
        y[k] = y[tr[k]];
        y[tr[k]] = t;
    }
    for (int i = 0; i < 6; ++i) x[i] = y[i];
}

// SE(3) exponential of (upsilon, omega): R = Rodrigues(omega),
// t = V upsilon, V = I + (1-cos)/th^2 W + (th - sin)/th^3 W^2 (series below 1e-4).
__device__ void se3_exp(const double *xi, double *T) {
    const double wx = xi[3], wy = xi[4], wz = xi[5];
    const double th2 = wx * wx + wy * wy + wz * wz;
    double A, B, C;  // sin/th, (1-cos)/th^2, (th-sin)/th^3
    if (th2 < 1e-8) {
        A = 1.0 - th2 / 6.0 + th2 * th2 / 120.0;
        B = 0.5 - th2 / 24.0 + th2 * th2 / 720.0;
        C = 1.0 / 6.0 - th2 / 120.0 + th2 * th2 / 5040.0;
    } else {
        const double th = sqrt(th2);
        double s, c;
        sincos(th, &s, &c);
        A = s / th;
        B = (1.0 - c) / th2;
        C = (th - s) / (th2 * th);
    }
    const double W[9] = {0, -wz, wy, wz, 0, -wx, -wy, wx, 0};
    double W2[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += W[i * 3 + k] * W[k * 3 + j];
            W2[i * 3 + j] = s;
        }
    double R[9], V[9];
    for (int i = 0; i < 9; ++i) {
        const double I = (i % 4 == 0) ? 1.0 : 0.0;
        R[i] = I + A * W[i] + B * W2[i];
        V[i] = I + B * W[i] + C * W2[i];
    }
    for (int i = 0; i < 3; ++i) {
        T[i * 4 + 0] = R[i * 3 + 0];
        T[i * 4 + 1] = R[i * 3 + 1];
        T[i * 4 + 2] = R[i * 3 + 2];
        T[i * 4 + 3] = V[i * 3 + 0] * xi[0] + V[i * 3 + 1] * xi[1] + V[i * 3 + 2] * xi[2];
    }
}

// T (row-major 3x4) = A * B
__device__ void pose_mul34(const double *A, const double *B, double *T) {
    double o[12];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            o[i * 4 + j] = A[i * 4 + 0] * B[0 * 4 + j] + A[i * 4 + 1] * B[1 * 4 + j] + A[i * 4 + 2] * B[2 * 4 + j];
        o[i * 4 + 3] = A[i * 4 + 0] * B[3] + A[i * 4 + 1] * B[7] + A[i * 4 + 2] * B[11] + A[i * 4 + 3];
    }
    for (int i = 0; i < 12; ++i) T[i] = o[i];
}

// Float copies of the estimate and R*K_l^-1 for every level.
__device__ void publish_estimate(GNState *st, const double Kd[kMaxLevels][4], int L) {
    const double *E = st->est;
    for (int i = 0; i < 12; ++i) st->Tf[i] = (float)E[i];
    for (int l = 0; l < L; ++l) {
        const double fx = Kd[l][0], fy = Kd[l][1], cx = Kd[l][2], cy = Kd[l][3];
        for (int i = 0; i < 3; ++i) {
            const double r0 = E[i * 4 + 0], r1 = E[i * 4 + 1], r2 = E[i * 4 + 2];
            st->RKinv[l][i * 3 + 0] = (float)(r0 / fx);
            st->RKinv[l][i * 3 + 1] = (float)(r1 / fy);
            st->RKinv[l][i * 3 + 2] = (float)(-r0 * cx / fx - r1 * cy / fy + r2);
        }
    }
}

__device__ void unpack_system(const double *v, double *H, double *b, double sH, double sb, bool add) {
    int k = 0;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 7; ++j) {
            const double val = v[k++];
            if (j == 6) {
                b[i] = (add ? b[i] : 0.0) + sb * val;
            } else {
                const double h = (add ? H[i * 6 + j] : 0.0) + sH * val;
                H[i * 6 + j] = h;
                H[j * 6 + i] = h;
            }
        }
}

// Thread 0 of the last CTA of the final pass of an iteration.
__device__ void gn_solve(const PassArgs &a) {
    GNState *st = a.st;
    double H[36], b[6];
    double residualSum, numResidual;
    const double *A = st->a_sums, *B = st->b_sums;
    if (a.mode == YAS_TRACK_RGBD) {
        unpack_system(B, H, b, 1.0, 1.0, false);
        unpack_system(A, H, b, 100.0, 10.0, true);
        residualSum = (double)(float)A[27];
        numResidual = (double)(float)A[29];
    } else if (a.mode == YAS_TRACK_RGB) {
        unpack_system(B, H, b, 1.0, 1.0, false);
        residualSum = (double)(float)B[27];
        numResidual = (double)(float)A[29];
    } else {
        unpack_system(A, H, b, 1.0, 1.0, false);
        residualSum = (double)(float)A[27];
        numResidual = (double)(float)A[28];
    }
    for (int i = 0; i < 36; ++i) st->H[i] = H[i];
    for (int i = 0; i < 6; ++i) st->b[i] = b[i];
    st->stats[0] = residualSum;
    st->stats[1] = numResidual;
    st->stats[2] = st->huber_th;
    st->stats[3] = A[28];
    if (a.no_update) return;
    const float error = sqrtf((float)residualSum) / ((float)numResidual + 6.0f);
    double upd[6];
    ldlt_solve6(H, b, upd);
    for (int i = 0; i < 6; ++i) st->last_update[i] = upd[i];
    if (isnan(upd[0])) {
        st->failed = 1;
        for (int i = 0; i < 12; ++i) st->best[i] = (i % 5 == 0) ? 1.0 : 0.0;
        return;
    }
    double E[12];
    se3_exp(upd, E);
    pose_mul34(E, st->est, st->est);
    if (a.first_of_level) st->last_error = (double)FLT_MAX;
    if ((double)error < st->last_error) {
        for (int i = 0; i < 12; ++i) st->best[i] = st->est[i];
        st->last_error = (double)error;
        st->n_success++;
    }
    st->n_iter++;
    st->level_of_last = a.level;
    publish_estimate(st, a.Kd, a.L);
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

__global__ void __launch_bounds__(kTrackThreads) gn_pass_a(PassArgs a) {
    GNState *st = a.st;
    if (*(volatile int *)&st->failed) return;
    __shared__ float sT[12], sRK[9];
    __shared__ double tot[32];
    if (threadIdx.x < 12) sT[threadIdx.x] = st->Tf[threadIdx.x];
    if (threadIdx.x < 9) sRK[threadIdx.x] = st->RKinv[a.level][threadIdx.x];
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
    if (!grid_reduce32(acc, a.partial, a.counter, tot)) return;
    if (threadIdx.x < 32) st->a_sums[threadIdx.x] = tot[threadIdx.x];
    if (threadIdx.x == 0) {
        // stddev of the photometric residuals (two-pass variance restated as
        // sum r^2 - (sum r)^2 / n in FP64), Huber threshold 4.685 * stddev.
        const double nn = tot[29], s = tot[30], s2 = tot[31];
        const double var = (s2 - s * s / nn) / (nn - 1.0);
        st->huber_th = (float)(4.685 * sqrt(var));
        if (a.mode == YAS_TRACK_ICP) gn_solve(a);
    }
}

__global__ void __launch_bounds__(kTrackThreads) gn_pass_b(PassArgs a) {
    GNState *st = a.st;
    if (*(volatile int *)&st->failed) return;
    __shared__ float sT[12], sRK[9];
    __shared__ double tot[32];
    if (threadIdx.x < 12) sT[threadIdx.x] = st->Tf[threadIdx.x];
    if (threadIdx.x < 9) sRK[threadIdx.x] = st->RKinv[a.level][threadIdx.x];
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
    if (!grid_reduce32(acc, a.partial, a.counter, tot)) return;
    if (threadIdx.x < 32) st->b_sums[threadIdx.x] = tot[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) gn_solve(a);
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
    a.counter = tr->counters;
    if (tr->hook) tr->hook(tr->hook_ctx, 10 + l);
    gn_pass_a<<<g, kTrackThreads, 0, s>>>(a);
    if (tr->mode & YAS_TRACK_RGB) {
        a.partial = tr->partialB;
        a.counter = tr->counters + 1;
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
    tr->partialA = (double *)grab((size_t)kMaxCtas * 32 * 8);
    tr->partialB = (double *)grab((size_t)kMaxCtas * 32 * 8);
    tr->counters = (unsigned *)grab(64);
    tr->state = (GNState *)grab(sizeof(GNState));
    tr->staging_bytes = (size_t)tr->w * tr->h * 4;
    tr->staging = grab(tr->staging_bytes);
    if (!tr->res4 || !tr->partialA || !tr->partialB || !tr->counters || !tr->state || !tr->staging)
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
