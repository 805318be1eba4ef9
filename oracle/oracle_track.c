/*
 * oracle_track.c — CPU restatement of the dense tracker and of the per-frame
 * session flow.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Reference files (paths relative to the reference project root):
 *   RGBDFusion/src/ImageProc.cu:7-286           gradients, inverse depth, pyr-down, vertex/normal maps
 *   RGBDFusion/src/RGBDTracking.cu:5-150        level intrinsics, pyramids, reference model
 *   RGBDFusion/src/RGBDTracking.cu:152-214      GetTransform schedule, error, acceptance, update
 *   RGBDFusion/src/RGBDTracking.cu:225-292      photometric step (residual, variance, Jacobian)
 *   RGBDFusion/include/TrackingUtils.h:45-220, 578-607   28-term layout, bilinear, weights
 *   RGBDFusion/src/RGBDTracking.cu:305-441      ICP step
 *   RGBDFusion/src/RGBDTracking.cu:521-545      H_rgb + 100 H_icp, b_rgb + 10 b_icp
 *   FullSystem/src/Tracking.cpp:139-197         first frame and tracked-frame flow
 *   FullSystem/src/System.cpp:43-65             RGB -> gray, u16 -> metres
 * Third-party arithmetic restated from its published definition:
 *   cv::cvtColor RGB2GRAY   BT.601 luma in 14-bit fixed point
 *   cv::cuda::pyrDown       separable [1 4 6 4 1]/16 Gaussian, reflect-101 border, even samples
 *   Eigen LDLT              left-looking LDL^T with diagonal pivoting, pseudo-inverse of D
 *   Sophus SE3::exp         Rodrigues rotation and left Jacobian V for the translation
 * Image buffers are stored in float as the reference's CV_32F buffers are;
 * residuals, Jacobians, reductions and the solve use `real`.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define MAXL 5

typedef struct {
    int w, h;
    float fx, fy, cx, cy, invfx, invfy;
    double dfx, dfy, dcx, dcy;
} lcam;

typedef struct {
    float *inten, *invd, *vmap, *nmap; /* vmap/nmap: 4 floats per pixel */
} lbufs;

struct orc_tracker {
    int w, h, L, mode;
    int iters[MAXL];
    lcam cam[MAXL];
    lbufs set[2][MAXL];
    float *gx[MAXL], *gy[MAXL];
    int cur;
    float angle_th, dist_th;
};

/* ------------------------------------------------------------ FP64 algebra */
void orc_ldlt_solve6(const double *Ain, const double *bin, double *x) {
    double A[36];
    int tr[6];
    memcpy(A, Ain, sizeof(A));
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
        if (k > 0) {
            double temp[6];
            for (int j = 0; j < k; ++j) temp[j] = A[j * 6 + j] * A[k * 6 + j];
            double s = 0;
            for (int j = 0; j < k; ++j) s += A[k * 6 + j] * temp[j];
            A[k * 6 + k] -= s;
            for (int i = k + 1; i < 6; ++i) {
                double t = 0;
                for (int j = 0; j < k; ++j) t += A[i * 6 + j] * temp[j];
                A[i * 6 + k] -= t;
            }
        }
        const double d = A[k * 6 + k];
        const int valid = fabs(d) > 0.0;
        if (k == 0 && !valid) {
            /* whole diagonal zero (or NaN): identity transpositions, solve as is */
            for (int j = 0; j < 6; ++j) tr[j] = j;
            break;
        }
        if (valid)
            for (int i = k + 1; i < 6; ++i) A[i * 6 + k] /= d;
    }
    double y[6];
    memcpy(y, bin, sizeof(y));
    for (int k = 0; k < 6; ++k) {
        double t = y[k];
        y[k] = y[tr[k]];
        y[tr[k]] = t;
    }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < i; ++j) y[i] -= A[i * 6 + j] * y[j];
    for (int i = 0; i < 6; ++i) y[i] = fabs(A[i * 6 + i]) > 1.0 / DBL_MAX ? y[i] / A[i * 6 + i] : 0.0;
    for (int i = 5; i >= 0; --i)
        for (int j = i + 1; j < 6; ++j) y[i] -= A[j * 6 + i] * y[j];
    for (int k = 5; k >= 0; --k) {
        double t = y[k];
        y[k] = y[tr[k]];
        y[tr[k]] = t;
    }
    memcpy(x, y, sizeof(y));
}

void orc_se3_exp(const double *xi, double *T) {
    const double wx = xi[3], wy = xi[4], wz = xi[5];
    const double th2 = wx * wx + wy * wy + wz * wz;
    double A, B, C;
    if (th2 < 1e-8) {
        A = 1.0 - th2 / 6.0 + th2 * th2 / 120.0;
        B = 0.5 - th2 / 24.0 + th2 * th2 / 720.0;
        C = 1.0 / 6.0 - th2 / 120.0 + th2 * th2 / 5040.0;
    } else {
        const double th = sqrt(th2);
        A = sin(th) / th;
        B = (1.0 - cos(th)) / th2;
        C = (th - sin(th)) / (th2 * th);
    }
    const double W[9] = {0, -wz, wy, wz, 0, -wx, -wy, wx, 0};
    double W2[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += W[i * 3 + k] * W[k * 3 + j];
            W2[i * 3 + j] = s;
        }
    for (int i = 0; i < 3; ++i) {
        double V[3];
        for (int j = 0; j < 3; ++j) {
            const double I = i == j ? 1.0 : 0.0;
            T[i * 4 + j] = I + A * W[i * 3 + j] + B * W2[i * 3 + j];
            V[j] = I + B * W[i * 3 + j] + C * W2[i * 3 + j];
        }
        T[i * 4 + 3] = V[0] * xi[0] + V[1] * xi[1] + V[2] * xi[2];
    }
}

static void mul34(const double *A, const double *B, double *T) {
    double o[12];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) o[i * 4 + j] = A[i * 4] * B[j] + A[i * 4 + 1] * B[4 + j] + A[i * 4 + 2] * B[8 + j];
        o[i * 4 + 3] = A[i * 4] * B[3] + A[i * 4 + 1] * B[7] + A[i * 4 + 2] * B[11] + A[i * 4 + 3];
    }
    memcpy(T, o, sizeof(o));
}

static void inv34(const double *A, double *T) {
    double o[12];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) o[i * 4 + j] = A[j * 4 + i];
        o[i * 4 + 3] = -((A[0 * 4 + i] * A[3] + A[1 * 4 + i] * A[7]) + A[2 * 4 + i] * A[11]);
    }
    memcpy(T, o, sizeof(o));
}

static void ident34(double *T) {
    for (int i = 0; i < 12; ++i) T[i] = (i % 5 == 0) ? 1.0 : 0.0;
}

/* ------------------------------------------------------------ images */
static int reflect101(int i, int n) {
    if (i < 0) i = -i;
    if (i >= n) i = 2 * (n - 1) - i;
    return i;
}

static void gray_to_level0(orc_tracker *t, const uint8_t *gray, float *inten, float *gx, float *gy) {
    const int w = t->w, h = t->h;
    for (int i = 0; i < w * h; ++i) inten[i] = (float)gray[i];
    if (!gx) return;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const int k = y * w + x;
            if (x < 1 || y < 1 || x > w - 2 || y > h - 2) {
                gx[k] = gy[k] = 0.0f;
            } else {
                gx[k] = (inten[k + 1] - inten[k - 1]) * 0.5f;
                gy[k] = (inten[k + w] - inten[k - w]) * 0.5f;
            }
        }
}

static void pyrdown(const float *src, int sw, int sh, float *dst, int dw, int dh) {
    static const float kk[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            float acc = 0.0f;
            for (int j = 0; j < 5; ++j) {
                const int cx = reflect101(2 * x + j - 2, sw);
                float col = 0.0f;
                for (int i = 0; i < 5; ++i) col += kk[i] * src[(size_t)reflect101(2 * y + i - 2, sh) * sw + cx];
                acc += kk[j] * col;
            }
            dst[y * dw + x] = acc;
        }
}

static void gradients(const float *src, int w, int h, float *gx, float *gy) {
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const int k = y * w + x;
            if (x < 1 || y < 1 || x > w - 2 || y > h - 2) {
                gx[k] = gy[k] = 0.0f;
            } else {
                gx[k] = (src[k + 1] - src[k - 1]) * 0.5f;
                gy[k] = (src[k + w] - src[k - w]) * 0.5f;
            }
        }
}

static void vertex_of(float invz, int x, int y, const lcam *c, float *v) {
    const float z = 1.0f / invz;
    if (invz > 0.0f && z < 3.0f) {
        v[0] = z * ((float)x - c->cx) * c->invfx;
        v[1] = z * ((float)y - c->cy) * c->invfy;
        v[2] = z;
        v[3] = 1.0f;
    } else {
        v[0] = v[1] = v[2] = 0.0f;
        v[3] = -1.0f;
    }
}

static void normals_from(const float *vmap, int w, int h, float *nmap) {
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            float *n = nmap + ((size_t)y * w + x) * 4;
            n[0] = n[1] = n[2] = 0.0f;
            n[3] = -1.0f;
            if (x == w - 1 || y == h - 1) continue;
            const float *v00 = vmap + ((size_t)y * w + x) * 4, *v01 = v00 + 4, *v10 = v00 + 4 * w;
            if (!(v00[3] > 0 && v01[3] > 0 && v10[3] > 0)) continue;
            const float a[3] = {v10[0] - v00[0], v10[1] - v00[1], v10[2] - v00[2]};
            const float b[3] = {v01[0] - v00[0], v01[1] - v00[1], v01[2] - v00[2]};
            float c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            const float nn = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
            if (nn > 0) {
                const float inv = 1.0f / sqrtf(nn);
                c[0] *= inv;
                c[1] *= inv;
                c[2] *= inv;
            }
            n[0] = c[0];
            n[1] = c[1];
            n[2] = c[2];
            n[3] = 1.0f;
        }
}

static void depth_levels(orc_tracker *t, const float *depth, lbufs *B) {
    for (int l = 0; l < t->L; ++l) {
        const lcam *c = &t->cam[l];
        if (l == 0) {
            for (int i = 0; i < c->w * c->h; ++i) {
                const float z = depth[i];
                B[0].invd[i] = (z > 0.2f && z < 8.0f) ? 1.0f / z : 0.0f;
            }
        } else {
            const lcam *p = &t->cam[l - 1];
            for (int y = 0; y < c->h; ++y)
                for (int x = 0; x < c->w; ++x)
                    B[l].invd[y * c->w + x] =
                        (x >= c->w - 1 || y >= c->h - 1) ? 0.0f : B[l - 1].invd[(size_t)(2 * y) * p->w + 2 * x];
        }
        for (int y = 0; y < c->h; ++y)
            for (int x = 0; x < c->w; ++x) vertex_of(B[l].invd[y * c->w + x], x, y, c, B[l].vmap + ((size_t)y * c->w + x) * 4);
        normals_from(B[l].vmap, c->w, c->h, B[l].nmap);
    }
}

orc_tracker *orc_tracker_create(int w, int h, const double *K, int levels, const int *iters, int mode) {
    orc_tracker *t = (orc_tracker *)calloc(1, sizeof(orc_tracker));
    t->w = w;
    t->h = h;
    t->L = levels;
    t->mode = mode;
    static const int def[MAXL] = {10, 5, 3, 3, 3};
    for (int l = 0; l < MAXL; ++l) {
        t->iters[l] = iters ? (l < levels ? iters[l] : 0) : def[l];
        const double s = (double)(1 << l);
        lcam *c = &t->cam[l];
        c->dfx = K[0] / s;
        c->dfy = K[4] / s;
        c->dcx = K[2] / s;
        c->dcy = K[5] / s;
        c->fx = (float)c->dfx;
        c->fy = (float)c->dfy;
        c->cx = (float)c->dcx;
        c->cy = (float)c->dcy;
        c->invfx = (float)(1.0 / c->dfx);
        c->invfy = (float)(1.0 / c->dfy);
        c->w = w >> l;
        c->h = h >> l;
    }
    for (int l = 0; l < levels; ++l) {
        const size_t n = (size_t)t->cam[l].w * t->cam[l].h;
        for (int s = 0; s < 2; ++s) {
            t->set[s][l].inten = (float *)calloc(n, 4);
            t->set[s][l].invd = (float *)calloc(n, 4);
            t->set[s][l].vmap = (float *)calloc(n * 4, 4);
            t->set[s][l].nmap = (float *)calloc(n * 4, 4);
        }
        t->gx[l] = (float *)calloc(n, 4);
        t->gy[l] = (float *)calloc(n, 4);
    }
    t->angle_th = sinf(20.f * 3.14159254f / 180.f);
    t->dist_th = 0.01f;
    return t;
}

void orc_tracker_destroy(orc_tracker *t) {
    if (!t) return;
    for (int l = 0; l < t->L; ++l) {
        for (int s = 0; s < 2; ++s) {
            free(t->set[s][l].inten);
            free(t->set[s][l].invd);
            free(t->set[s][l].vmap);
            free(t->set[s][l].nmap);
        }
        free(t->gx[l]);
        free(t->gy[l]);
    }
    free(t);
}

/* SetReferenceImage / SetTrackingImage (RGBDTracking.cu:66-116) */
void orc_tracker_set_image(orc_tracker *t, const uint8_t *gray, int reference) {
    lbufs *B = t->set[reference ? 1 - t->cur : t->cur];
    gray_to_level0(t, gray, B[0].inten, reference ? NULL : t->gx[0], reference ? NULL : t->gy[0]);
    for (int l = 1; l < t->L; ++l) {
        pyrdown(B[l - 1].inten, t->cam[l - 1].w, t->cam[l - 1].h, B[l].inten, t->cam[l].w, t->cam[l].h);
        if (!reference) gradients(B[l].inten, t->cam[l].w, t->cam[l].h, t->gx[l], t->gy[l]);
    }
}

/* SetReferenceDepth / SetTrackingDepth (RGBDTracking.cu:80-138) */
void orc_tracker_set_depth(orc_tracker *t, const float *depth, int reference) {
    depth_levels(t, depth, t->set[reference ? 1 - t->cur : t->cur]);
}

/* SetReferenceModel (RGBDTracking.cu:140-150) with the float4 nearest pyr-down. */
void orc_tracker_set_model(orc_tracker *t, const float *vmap) {
    lbufs *B = t->set[1 - t->cur];
    memcpy(B[0].vmap, vmap, sizeof(float) * 4 * t->w * t->h);
    normals_from(B[0].vmap, t->w, t->h, B[0].nmap);
    for (int l = 1; l < t->L; ++l) {
        const lcam *c = &t->cam[l], *p = &t->cam[l - 1];
        for (int y = 0; y < c->h; ++y)
            for (int x = 0; x < c->w; ++x) {
                float *v = B[l].vmap + ((size_t)y * c->w + x) * 4;
                if (x >= c->w - 1 || y >= c->h - 1) {
                    v[0] = v[1] = v[2] = 0.0f;
                    v[3] = -1.0f;
                } else {
                    memcpy(v, B[l - 1].vmap + ((size_t)(2 * y) * p->w + 2 * x) * 4, 16);
                }
            }
        normals_from(B[l].vmap, c->w, c->h, B[l].nmap);
    }
}

void orc_tracker_swap(orc_tracker *t) { t->cur = 1 - t->cur; }

void orc_tracker_level(const orc_tracker *t, int level, int which, float *out) {
    const lbufs *c = &t->set[t->cur][level], *r = &t->set[1 - t->cur][level];
    const size_t n = (size_t)t->cam[level].w * t->cam[level].h;
    const float *src;
    size_t k = 1;
    switch (which) {
        case 0: src = c->inten; break;
        case 1: src = t->gx[level]; break;
        case 2: src = t->gy[level]; break;
        case 3: src = c->invd; break;
        case 4: src = c->vmap; k = 4; break;
        case 5: src = c->nmap; k = 4; break;
        case 6: src = r->inten; break;
        case 7: src = r->invd; break;
        case 8: src = r->vmap; k = 4; break;
        default: src = r->nmap; k = 4; break;
    }
    memcpy(out, src, sizeof(float) * n * k);
}

/* ------------------------------------------------------------ GN step */
static real bilinear(const float *m, int w, real x, real y) {
    const int u = (int)floor(x), v = (int)floor(y);
    const real cx = x - u, cy = y - v;
    const float *r0 = m + (size_t)v * w + u, *r1 = r0 + w;
    return ((real)r0[0] * (1 - cx) + (real)r0[1] * cx) * (1 - cy) + ((real)r1[0] * (1 - cx) + (real)r1[1] * cx) * cy;
}

/* Discrete decisions of the tracker, in IEEE FP32 at the FP32 pose Tf (the
 * reference casts its SE3d to float for the kernels), one rounding per
 * operation in the device code's fixed order: which reference pixels
 * project inside the current image (se3StepRGBFunctor's bounds,
 * TrackingUtils.h:73-150), which model point pairs with which current pixel
 * and passes the ICP gates (IcpStepFunctor::ProjectPoint,
 * RGBDTracking.cu:326-358), and the point-to-plane residual whose squares
 * GetTransform's error sums.  Coordinates are tested as floats before they
 * are converted, so NaN and infinite projections are outside. */
static float dot3f(float a0, float a1, float a2, float b0, float b1, float b2) {
    const float p0 = a0 * b0, p1 = a1 * b1, p2 = a2 * b2;
    const float s = p0 + p1;
    return s + p2;
}

/* R K^-1 in FP32 from the FP32 pose (the device forms it the same way). */
static void rkinv_f(const float *Tf, const lcam *c, float *RK) {
    const float cxi = c->cx * c->invfx, cyi = c->cy * c->invfy;
    for (int i = 0; i < 3; ++i) {
        RK[i * 3 + 0] = Tf[i * 4 + 0] * c->invfx;
        RK[i * 3 + 1] = Tf[i * 4 + 1] * c->invfy;
        const float a = Tf[i * 4 + 0] * cxi, bq = Tf[i * 4 + 1] * cyi;
        const float d = Tf[i * 4 + 2] - a;
        RK[i * 3 + 2] = d - bq;
    }
}

/* Reference pixel (x, y) at depth z warped by Tf (TransformReferencePoint,
 * ImageProc.cu:42-78): (RK (x, y, 1)) z + t. */
static void warp_f(const float *RK, const float *Tf, int x, int y, float z, float *p) {
    const float fx = (float)x, fy = (float)y;
    for (int i = 0; i < 3; ++i) {
        const float a = RK[i * 3] * fx, bq = RK[i * 3 + 1] * fy;
        const float s = a + bq;
        const float s2 = s + RK[i * 3 + 2];
        const float m = s2 * z;
        p[i] = m + Tf[i * 4 + 3];
    }
}

static int rgb_project_f(const lcam *c, const float *p, float *u, float *v) {
    const float ax = c->fx * p[0], ay = c->fy * p[1];
    const float qx = ax / p[2], qy = ay / p[2];
    *u = qx + c->cx;
    *v = qy + c->cy;
    return *u > 0.0f && *v > 0.0f && *u < (float)(c->w - 1) && *v < (float)(c->h - 1);
}

/* Model pixel k: returns the current pixel index it pairs with and passes
 * the gates, or -1; rf = n . (v_c - v_m) in FP32. */
static int icp_match_f(const orc_tracker *t, const lcam *c, const lbufs *cb, const lbufs *rb, const float *Tf, int k,
                       float *rf) {
    const float *vm = rb->vmap + (size_t)k * 4;
    if (!(vm[3] >= 0.0f)) return -1;
    float vl[3], nl[3];
    for (int i = 0; i < 3; ++i) vl[i] = dot3f(Tf[i * 4], Tf[i * 4 + 1], Tf[i * 4 + 2], vm[0], vm[1], vm[2]) + Tf[i * 4 + 3];
    const float invz = 1.0f / vl[2];
    const float ax = c->fx * vl[0], ay = c->fy * vl[1];
    const float bx = ax * invz, by = ay * invz;
    const float cxs = bx + c->cx, cys = by + c->cy;
    const float fu = floorf(cxs + 0.5f), fv = floorf(cys + 0.5f);
    if (!(fu >= 0.0f && fv >= 0.0f && fu < (float)c->w && fv < (float)c->h)) return -1;
    const int q = (int)fv * c->w + (int)fu;
    const float *vc = cb->vmap + (size_t)q * 4;
    if (!(vc[3] >= 0.0f)) return -1;
    const float *nm = rb->nmap + (size_t)k * 4, *nc = cb->nmap + (size_t)q * 4;
    for (int i = 0; i < 3; ++i) nl[i] = dot3f(Tf[i * 4], Tf[i * 4 + 1], Tf[i * 4 + 2], nm[0], nm[1], nm[2]);
    const float dx = vl[0] - vc[0], dy = vl[1] - vc[1], dz = vl[2] - vc[2];
    const float dist = sqrtf(dot3f(dx, dy, dz, dx, dy, dz));
    const float a0 = nc[1] * nl[2], a1 = nc[2] * nl[1], b0 = nc[2] * nl[0], b1 = nc[0] * nl[2];
    const float c0 = nc[0] * nl[1], c1 = nc[1] * nl[0];
    const float cx_ = a0 - a1, cy_ = b0 - b1, cz_ = c0 - c1;
    const float angle = sqrtf(dot3f(cx_, cy_, cz_, cx_, cy_, cz_));
    if (!(angle < t->angle_th && dist <= t->dist_th && nm[3] > 0 && nc[3] > 0)) return -1;
    *rf = dot3f(nl[0], nl[1], nl[2], vc[0] - vl[0], vc[1] - vl[1], vc[2] - vl[2]);
    return q;
}

/* One linearisation at T on level l: sums[0..27] ICP products (27 = r^2),
 * sums[28] ICP count; rgb[0..27] weighted photometric products, rgbn count;
 * returns huber threshold. */
static void linearise(orc_tracker *t, int l, const double *T, double *H, double *b, double *stats) {
    const lcam *c = &t->cam[l];
    const lbufs *cb = &t->set[t->cur][l], *rb = &t->set[1 - t->cur][l];
    const int n = c->w * c->h;
    float Tf[12], RKf[9];
    for (int i = 0; i < 12; ++i) Tf[i] = (float)T[i];
    rkinv_f(Tf, c, RKf);
    /* R K^-1 (TransformReferencePoint, ImageProc.cu:86-101) */
    double RK[9];
    for (int i = 0; i < 3; ++i) {
        RK[i * 3 + 0] = T[i * 4 + 0] / c->dfx;
        RK[i * 3 + 1] = T[i * 4 + 1] / c->dfy;
        RK[i * 3 + 2] = -T[i * 4 + 0] * c->dcx / c->dfx - T[i * 4 + 1] * c->dcy / c->dfy + T[i * 4 + 2];
    }
    double icp[29] = {0}, rgb[28] = {0};
    double rsum = 0, rn = 0, th = 0;
    const int do_rgb = (t->mode & 1) != 0, do_icp = (t->mode & 2) != 0;
    real *res = NULL;
    real *pts = NULL;
    if (do_rgb) {
        res = (real *)malloc(sizeof(real) * 4 * n);
        pts = (real *)malloc(sizeof(real) * 3 * n);
        for (int k = 0; k < n; ++k) {
            const int y = k / c->w, x = k - y * c->w;
            real r = 0, gx = 0, gy = 0;
            int ok = 0;
            const float zinv = rb->invd[k];
            if (zinv > 0.0f) {
                const float zf = 1.0f / zinv;
                const real z = (real)zf;
                real p[3];
                for (int i = 0; i < 3; ++i) p[i] = (RK[i * 3] * x + RK[i * 3 + 1] * y + RK[i * 3 + 2]) * z + T[i * 4 + 3];
                pts[3 * k] = p[0];
                pts[3 * k + 1] = p[1];
                pts[3 * k + 2] = p[2];
                /* inside or outside, and where the current image is sampled:
                 * the FP32 decision at Tf */
                float pf[3], uf, vf;
                warp_f(RKf, Tf, x, y, zf, pf);
                if (rgb_project_f(c, pf, &uf, &vf)) {
                    const real u = (real)uf, v = (real)vf;
                    r = bilinear(cb->inten, c->w, u, v) - (real)rb->inten[k];
                    gx = bilinear(t->gx[l], c->w, u, v);
                    gy = bilinear(t->gy[l], c->w, u, v);
                    ok = (gx * gx + gy * gy) > 0 && isfinite(r);
                }
            }
            res[4 * k] = r;
            res[4 * k + 1] = gx;
            res[4 * k + 2] = gy;
            res[4 * k + 3] = ok ? 1 : -1;
            if (ok) {
                rsum += r;
                rn += 1;
            }
        }
        /* VarianceEstimator (TrackingUtils.h:578-607), two passes */
        const double mean = rsum / rn;
        double ss = 0;
        for (int k = 0; k < n; ++k)
            if (res[4 * k + 3] > 0) ss += (res[4 * k] - mean) * (res[4 * k] - mean);
        th = 4.685 * sqrt(ss / (rn - 1));
        /* se3StepRGBFunctor (TrackingUtils.h:163-197) */
        for (int k = 0; k < n; ++k) {
            if (!(res[4 * k + 3] > 0)) continue;
            const real *p = pts + 3 * k;
            const real zInv = 1 / p[2];
            const real r = res[4 * k], gxv = res[4 * k + 1], gyv = res[4 * k + 2];
            real wt = 1;
            if (fabs(r) > th) wt = th / fabs(r);
            real row[7];
            row[0] = gxv * c->fx * zInv;
            row[1] = gyv * c->fy * zInv;
            row[2] = -(row[0] * p[0] + row[1] * p[1]) * zInv;
            row[3] = row[2] * p[1] - gyv * c->fy;
            row[4] = -row[2] * p[0] + gxv * c->fx;
            row[5] = -row[0] * p[1] + row[1] * p[0];
            row[6] = -r;
            int q = 0;
            for (int i = 0; i < 7; ++i)
                for (int j = i; j < 7; ++j) rgb[q++] += wt * row[i] * row[j];
        }
        free(res);
        free(pts);
    }
    if (do_icp) {
        /* IcpStepFunctor (RGBDTracking.cu:432-488) */
        for (int k = 0; k < n; ++k) {
            /* the pairing and the gates: the FP32 decision at Tf */
            float rf = 0.0f;
            const int q = icp_match_f(t, c, cb, rb, Tf, k, &rf);
            if (q < 0) continue;
            const float *vm = rb->vmap + (size_t)k * 4;
            const float *vc = cb->vmap + (size_t)q * 4, *nm = rb->nmap + (size_t)k * 4;
            real vl[3], nl[3];
            for (int i = 0; i < 3; ++i) vl[i] = T[i * 4] * vm[0] + T[i * 4 + 1] * vm[1] + T[i * 4 + 2] * vm[2] + T[i * 4 + 3];
            for (int i = 0; i < 3; ++i) nl[i] = T[i * 4] * nm[0] + T[i * 4 + 1] * nm[1] + T[i * 4 + 2] * nm[2];
            real row[7];
            row[0] = nl[0];
            row[1] = nl[1];
            row[2] = nl[2];
            row[3] = vl[1] * nl[2] - vl[2] * nl[1];
            row[4] = vl[2] * nl[0] - vl[0] * nl[2];
            row[5] = vl[0] * nl[1] - vl[1] * nl[0];
            row[6] = nl[0] * (vc[0] - vl[0]) + nl[1] * (vc[1] - vl[1]) + nl[2] * (vc[2] - vl[2]);
            int qq = 0;
            for (int i = 0; i < 7; ++i)
                for (int j = i; j < 7; ++j, ++qq)
                    if (qq < 27) icp[qq] += row[i] * row[j];
            /* the error's sum of squares: the FP32 residual's rounded squares */
            icp[27] += (double)(rf * rf);
            icp[28] += 1;
        }
    }
    /* RankUpdateHessian<6,7> and the RGB+ICP combination */
    for (int i = 0; i < 36; ++i) H[i] = 0;
    for (int i = 0; i < 6; ++i) b[i] = 0;
    const double sH = t->mode == 3 ? 100.0 : 1.0, sb = t->mode == 3 ? 10.0 : 1.0;
    int q = 0;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 7; ++j, ++q) {
            double v = 0, vb = 0;
            if (do_rgb) {
                v += rgb[q];
                vb += rgb[q];
            }
            if (do_icp) {
                v += sH * icp[q];
                vb += sb * icp[q];
            }
            if (j == 6)
                b[i] = vb;
            else
                H[i * 6 + j] = H[j * 6 + i] = v;
        }
    double residualSum, numResidual;
    if (t->mode == 3) {
        residualSum = icp[27];
        numResidual = rn;
    } else if (t->mode == 1) {
        residualSum = rgb[27];
        numResidual = rn;
    } else {
        residualSum = icp[27];
        numResidual = icp[28];
    }
    stats[0] = residualSum;
    stats[1] = numResidual;
    stats[2] = th;
    stats[3] = icp[28];
}

void orc_tracker_compute_step(orc_tracker *t, int level, const double *T, double *H, double *b, double *stats) {
    linearise(t, level, T, H, b, stats);
}

int orc_tracker_get_transform(orc_tracker *t, const double *init, int swap, double *out) {
    double est[12], best[12];
    memcpy(est, init, sizeof(est));
    memcpy(best, init, sizeof(best));
    for (int l = t->L - 1; l >= 0; --l) {
        float last_error = FLT_MAX;
        for (int it = 0; it < t->iters[l]; ++it) {
            double H[36], b[6], st[4], upd[6], E[12];
            linearise(t, l, est, H, b, st);
            /* float error = sqrt(residualSum) / (numResidual + 6), in FP32 as
             * the reference computes and compares it */
            const float error = sqrtf((float)st[0]) / ((float)st[1] + 6.0f);
            orc_ldlt_solve6(H, b, upd);
            if (isnan(upd[0])) {
                ident34(out);
                return 6;
            }
            orc_se3_exp(upd, E);
            mul34(E, est, est);
            if (error < last_error) {
                memcpy(best, est, sizeof(best));
                last_error = error;
            }
        }
    }
    if (swap) orc_tracker_swap(t);
    memcpy(out, best, sizeof(best));
    return 0;
}

/* ------------------------------------------------------------ session */
struct orc_session {
    int w, h;
    float K[4];
    float depth_scale, max_step;
    orc_map *map;
    orc_tracker *tr;
    double Tcm[12];
    int frames;
    float *depth_m;
    uint8_t *gray;
    float *vmap;
};

orc_session *orc_session_create(int w, int h, const float *K, float voxel_size, float trunc, int levels,
                                const int *iters, int mode, float depth_scale, float max_step) {
    orc_session *s = (orc_session *)calloc(1, sizeof(orc_session));
    s->w = w;
    s->h = h;
    memcpy(s->K, K, sizeof(s->K));
    s->depth_scale = depth_scale;
    s->max_step = max_step;
    s->map = orc_map_create(voxel_size, trunc, 0.1f, 3.0f, 255);
    const double Kd[9] = {K[0], 0, K[2], 0, K[1], K[3], 0, 0, 1};
    s->tr = orc_tracker_create(w, h, Kd, levels, iters, mode);
    ident34(s->Tcm);
    s->depth_m = (float *)malloc(sizeof(float) * w * h);
    s->gray = (uint8_t *)malloc((size_t)w * h);
    s->vmap = (float *)malloc(sizeof(float) * 4 * w * h);
    return s;
}

void orc_session_destroy(orc_session *s) {
    if (!s) return;
    orc_map_destroy(s->map);
    orc_tracker_destroy(s->tr);
    free(s->depth_m);
    free(s->gray);
    free(s->vmap);
    free(s);
}

orc_map *orc_session_map(orc_session *s) { return s->map; }
orc_tracker *orc_session_tracker(orc_session *s) { return s->tr; }

int orc_session_frame(orc_session *s, const uint8_t *rgb, const uint16_t *depth, double *out_Tcm) {
    const int n = s->w * s->h;
    for (int i = 0; i < n; ++i) {
        const int r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
        s->gray[i] = (uint8_t)((r * 4899 + g * 9617 + b * 1868 + 8192) >> 14);
        s->depth_m[i] = (float)depth[i] * s->depth_scale;
    }
    int status = 0;
    if (s->frames == 0) {
        orc_tracker_set_image(s->tr, s->gray, 1);
        orc_tracker_set_depth(s->tr, s->depth_m, 1);
        orc_map_fuse(s->map, s->depth_m, s->w, s->h, s->K, s->Tcm);
    } else {
        orc_raycast(s->map, s->w, s->h, s->K, s->Tcm, s->vmap, NULL, NULL);
        orc_tracker_set_model(s->tr, s->vmap);
        orc_tracker_set_image(s->tr, s->gray, 0);
        orc_tracker_set_depth(s->tr, s->depth_m, 0);
        double I[12], DT[12];
        ident34(I);
        status = orc_tracker_get_transform(s->tr, I, 1, DT);
        if (status == 0) {
            /* the device pipeline swaps the pyramids every frame */
        } else {
            orc_tracker_swap(s->tr);
        }
        if (status == 0) {
            const double tn = sqrt(DT[3] * DT[3] + DT[7] * DT[7] + DT[11] * DT[11]);
            if (!(tn <= (double)s->max_step)) {
                status = 7;
            } else {
                double Di[12];
                inv34(DT, Di);
                mul34(s->Tcm, Di, s->Tcm);
                orc_map_fuse(s->map, s->depth_m, s->w, s->h, s->K, s->Tcm);
            }
        }
    }
    s->frames++;
    if (out_Tcm) memcpy(out_Tcm, s->Tcm, sizeof(double) * 12);
    return status;
}
