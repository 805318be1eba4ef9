/*
 * oracle_map.c — CPU restatement of the voxel-hash TSDF map, the raycaster
 * and marching cubes.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Reference files (paths relative to the reference project root):
 *   RGBDFusion/utils/VoxelStructUtils.h:6-147   packing, coordinates, visibility
 *   RGBDFusion/src/VoxelMap.cu:517-652          block allocation by 3-D line tracing
 *   RGBDFusion/src/VoxelMap.cu:654-717          visible-block selection
 *   RGBDFusion/src/VoxelMap.cu:719-786          TSDF integration
 *   RGBDFusion/src/RayTraceEngine.cu:58-410     z-range tiles and ray marching
 *   RGBDFusion/src/MeshEngine.cu:43-268         marching cubes
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

struct orc_map {
    float vs, trunc, dmin, dmax;
    int max_w;
    int q16; /* storage of the reference's int16 sdf (orc_map_set_storage) */
    int n, cap;
    int *coords;
    real *sdf;
    int *wt;
    int hcap;
    unsigned long long *hkey;
    int *hval;
};

#define EMPTY_KEY (~0ull)

static unsigned long long pack(int x, int y, int z) {
    return ((unsigned long long)(x & 0x1FFFFF) << 42) | ((unsigned long long)(y & 0x1FFFFF) << 21) |
           (unsigned long long)(z & 0x1FFFFF);
}

static unsigned long long mix(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

static int find_block(const orc_map *m, int x, int y, int z) {
    unsigned long long k = pack(x, y, z);
    unsigned s = (unsigned)mix(k) & (unsigned)(m->hcap - 1);
    for (;;) {
        if (m->hkey[s] == k) return m->hval[s];
        if (m->hkey[s] == EMPTY_KEY) return -1;
        s = (s + 1) & (unsigned)(m->hcap - 1);
    }
}

static void rehash(orc_map *m, int ncap) {
    unsigned long long *ok = m->hkey;
    int *ov = m->hval, oc = m->hcap;
    m->hcap = ncap;
    m->hkey = (unsigned long long *)malloc(sizeof(unsigned long long) * ncap);
    m->hval = (int *)malloc(sizeof(int) * ncap);
    for (int i = 0; i < ncap; ++i) m->hkey[i] = EMPTY_KEY;
    for (int i = 0; i < oc; ++i) {
        if (ok[i] == EMPTY_KEY) continue;
        unsigned s = (unsigned)mix(ok[i]) & (unsigned)(ncap - 1);
        while (m->hkey[s] != EMPTY_KEY) s = (s + 1) & (unsigned)(ncap - 1);
        m->hkey[s] = ok[i];
        m->hval[s] = ov[i];
    }
    free(ok);
    free(ov);
}

static int insert_block(orc_map *m, int x, int y, int z) {
    int f = find_block(m, x, y, z);
    if (f >= 0) return f;
    if (2 * (m->n + 1) > m->hcap) rehash(m, m->hcap * 2);
    if (m->n == m->cap) {
        m->cap *= 2;
        m->coords = (int *)realloc(m->coords, sizeof(int) * 3 * m->cap);
        m->sdf = (real *)realloc(m->sdf, sizeof(real) * 512 * (size_t)m->cap);
        m->wt = (int *)realloc(m->wt, sizeof(int) * 512 * (size_t)m->cap);
    }
    int idx = m->n++;
    m->coords[3 * idx] = x;
    m->coords[3 * idx + 1] = y;
    m->coords[3 * idx + 2] = z;
    for (int i = 0; i < 512; ++i) {
        m->sdf[(size_t)idx * 512 + i] = 0;
        m->wt[(size_t)idx * 512 + i] = 0;
    }
    unsigned long long k = pack(x, y, z);
    unsigned s = (unsigned)mix(k) & (unsigned)(m->hcap - 1);
    while (m->hkey[s] != EMPTY_KEY) s = (s + 1) & (unsigned)(m->hcap - 1);
    m->hkey[s] = k;
    m->hval[s] = idx;
    return idx;
}

orc_map *orc_map_create(float voxel_size, float trunc, float depth_min, float depth_max, int max_weight) {
    orc_map *m = (orc_map *)calloc(1, sizeof(orc_map));
    m->vs = voxel_size;
    m->trunc = trunc;
    m->dmin = depth_min;
    m->dmax = depth_max;
    m->max_w = max_weight;
    m->cap = 1024;
    m->coords = (int *)malloc(sizeof(int) * 3 * m->cap);
    m->sdf = (real *)malloc(sizeof(real) * 512 * (size_t)m->cap);
    m->wt = (int *)malloc(sizeof(int) * 512 * (size_t)m->cap);
    m->hcap = 4096;
    m->hkey = (unsigned long long *)malloc(sizeof(unsigned long long) * m->hcap);
    m->hval = (int *)malloc(sizeof(int) * m->hcap);
    for (int i = 0; i < m->hcap; ++i) m->hkey[i] = EMPTY_KEY;
    return m;
}

void orc_map_destroy(orc_map *m) {
    if (!m) return;
    free(m->coords);
    free(m->sdf);
    free(m->wt);
    free(m->hkey);
    free(m->hval);
    free(m);
}

int orc_map_num_blocks(const orc_map *m) { return m->n; }

/* ------------------------------------------------------------ FP32 canon */
typedef struct {
    float r[9];
    float t[3];
} rig32;

static rig32 rig_from(const double *T) {
    rig32 o;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) o.r[i * 3 + j] = (float)T[i * 4 + j];
        o.t[i] = (float)T[i * 4 + 3];
    }
    return o;
}

/* inverse [R^T | -R^T t], computed in double and rounded once */
static rig32 rig_inv_from(const double *T) {
    rig32 o;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) o.r[i * 3 + j] = (float)T[j * 4 + i];
        o.t[i] = (float)(-((T[0 * 4 + i] * T[3] + T[1 * 4 + i] * T[7]) + T[2 * 4 + i] * T[11]));
    }
    return o;
}

static void rig_apply(const rig32 *T, float x, float y, float z, float *o) {
    o[0] = ((T->r[0] * x + T->r[1] * y) + T->r[2] * z) + T->t[0];
    o[1] = ((T->r[3] * x + T->r[4] * y) + T->r[5] * z) + T->t[1];
    o[2] = ((T->r[6] * x + T->r[7] * y) + T->r[8] * z) + T->t[2];
}

static int f2i_floor(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT_MIN;
    return (int)floorf(x);
}

static int floor_div8(int v) { return v >= 0 ? v / 8 : -((-v + 7) / 8); }

/* UnProjectWorld -> WorldPtToVoxelPos -> VoxelPosToBlockPos (VoxelStructUtils.h:28-110) */
static void ray_block(float invfx, float invfy, float cx, float cy, const rig32 *T, float vs, int x, int y,
                      float z, int b[3]) {
    float p[3], q[3];
    p[0] = (invfx * ((float)x - cx)) * z;
    p[1] = (invfy * ((float)y - cy)) * z;
    p[2] = z;
    rig_apply(T, p[0], p[1], p[2], q);
    for (int i = 0; i < 3; ++i) b[i] = floor_div8(f2i_floor(q[i] / vs));
}

/* Allocation (VoxelMap.cu:549-651): 3-D Bresenham over the block coordinates
 * between depth - trunc/2 and depth + trunc/2 (clamped to the depth range). */
void orc_map_allocate(orc_map *m, const float *depth, int w, int h, const float *K, const double *Tcm) {
    const rig32 T = rig_from(Tcm);
    const float invfx = (float)(1.0 / (double)K[0]), invfy = (float)(1.0 / (double)K[1]);
    const float half = m->trunc * 0.5f;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const float dist = depth[(size_t)y * w + x];
            if (isnan(dist) || dist < m->dmin || dist > m->dmax) continue;
            const float dnear = fmaxf(m->dmin, dist - half);
            const float dfar = fminf(m->dmax, dist + half);
            if (dnear >= dfar) continue;
            int s[3], e[3];
            ray_block(invfx, invfy, K[2], K[3], &T, m->vs, x, y, dnear, s);
            ray_block(invfx, invfy, K[2], K[3], &T, m->vs, x, y, dfar, e);
            int inc[3], ad[3], d2[3], cur[3];
            for (int i = 0; i < 3; ++i) {
                int d = e[i] - s[i];
                inc[i] = d < 0 ? -1 : 1;
                ad[i] = d < 0 ? -d : d;
                d2[i] = ad[i] << 1;
                cur[i] = s[i];
            }
            int M, a1, a2;
            if (ad[0] >= ad[1] && ad[0] >= ad[2]) {
                M = 0; a1 = 1; a2 = 2;
            } else if (ad[1] >= ad[0] && ad[1] >= ad[2]) {
                M = 1; a1 = 0; a2 = 2;
            } else {
                M = 2; a1 = 1; a2 = 0;
            }
            int err1 = d2[a1] - 1, err2 = d2[a2] - 1;
            insert_block(m, cur[0], cur[1], cur[2]);
            for (int i = 0; i < ad[M]; ++i) {
                if (err1 > 0) {
                    cur[a1] += inc[a1];
                    err1 -= d2[M];
                }
                if (err2 > 0) {
                    cur[a2] += inc[a2];
                    err2 -= d2[M];
                }
                err1 += d2[a1];
                err2 += d2[a2];
                cur[M] += inc[M];
                insert_block(m, cur[0], cur[1], cur[2]);
            }
        }
}

/* CheckBlockVisibility (VoxelStructUtils.h:112-147) */
static int block_visible(const orc_map *m, const float *K, int cols, int rows, const rig32 *Tinv, int bx, int by,
                         int bz) {
    const float scale = m->vs * 8.0f;
    for (int c = 0; c < 8; ++c) {
        float wpt[3] = {(float)(bx + (c & 1)) * scale, (float)(by + ((c >> 1) & 1)) * scale,
                        (float)(bz + ((c >> 2) & 1)) * scale};
        float p[3];
        rig_apply(Tinv, wpt[0], wpt[1], wpt[2], p);
        const float u = (K[0] * p[0]) / p[2] + K[2];
        const float v = (K[1] * p[1]) / p[2] + K[3];
        if (!(u < 0.0f || v < 0.0f || u > (float)(cols - 1) || v > (float)(rows - 1) || p[2] < m->dmin ||
              p[2] > m->dmax))
            return 1;
    }
    return 0;
}

static int collect_visible(const orc_map *m, int cols, int rows, const float *K, const double *Tcm, int *list) {
    const rig32 Tinv = rig_inv_from(Tcm);
    int n = 0;
    for (int i = 0; i < m->n; ++i)
        if (block_visible(m, K, cols, rows, &Tinv, m->coords[3 * i], m->coords[3 * i + 1], m->coords[3 * i + 2]))
            list[n++] = i;
    return n;
}

int orc_map_visible(orc_map *m, int cols, int rows, const float *K, const double *Tcm, int *coords, int cap) {
    int *list = (int *)malloc(sizeof(int) * (m->n + 1));
    int n = collect_visible(m, cols, rows, K, Tcm, list);
    for (int i = 0; i < n && i < cap; ++i) {
        coords[3 * i] = m->coords[3 * list[i]];
        coords[3 * i + 1] = m->coords[3 * list[i] + 1];
        coords[3 * i + 2] = m->coords[3 * list[i] + 2];
    }
    free(list);
    return n;
}

/* A written sdf as the map keeps it: as computed, or with the reference's
 * int16 storage (PackFloat / UnPackFloat, VoxelStructUtils.h:6-14): the
 * FP32 product s * 32767 truncated toward zero, read back as q / 32767. */
static real stored(const orc_map *m, real s) {
    if (!m->q16) return s;
    const float p = (float)s * 32767.0f;
    int q = (int)p;
    if (q > 32767) q = 32767;
    if (q < -32767) q = -32767;
    return (real)((float)q / 32767.0f);
}

void orc_map_set_storage(orc_map *m, int int16_sdf) { m->q16 = int16_sdf != 0; }

/* Integration (VoxelMap.cu:738-785): pixel selection and gates in FP32, the
 * running weighted average in `real`. */
/* sign = +1: DepthFusionFunctor (VoxelMap.cu:719-786); sign = -1: the same
 * observation removed (s <- (s w - d) / (w - 1), w <- w - 1; w = 1 -> unobserved). */
static void integrate(orc_map *m, const float *depth, int w, int h, const float *K, const double *Tcm, const int *list,
                      int nvis, int sign) {
    const rig32 Tinv = rig_inv_from(Tcm);
    const float ntrunc = -m->trunc;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int j = 0; j < nvis; ++j) {
        const int b = list[j];
        const int bx = m->coords[3 * b], by = m->coords[3 * b + 1], bz = m->coords[3 * b + 2];
        for (int lz = 0; lz < 8; ++lz)
            for (int ly = 0; ly < 8; ++ly)
                for (int lx = 0; lx < 8; ++lx) {
                    const float wx = (float)(bx * 8 + lx) * m->vs;
                    const float wy = (float)(by * 8 + ly) * m->vs;
                    const float wz = (float)(bz * 8 + lz) * m->vs;
                    float p[3];
                    rig_apply(&Tinv, wx, wy, wz, p);
                    const int u = f2i_floor(((K[0] * p[0]) / p[2] + K[2]) + 0.5f);
                    const int v = f2i_floor(((K[1] * p[1]) / p[2] + K[3]) + 0.5f);
                    if (u < 0 || v < 0 || u > w - 1 || v > h - 1) continue;
                    const float dist = depth[(size_t)v * w + u];
                    if (isnan(dist) || dist > m->dmax || dist < m->dmin) continue;
                    const float sdf32 = dist - p[2];
                    if (sdf32 < ntrunc) continue;
                    real sdf = ((real)dist - (real)p[2]) / (real)m->trunc;
                    if (sdf > 1) sdf = 1;
                    const size_t k = (size_t)b * 512 + lz * 64 + ly * 8 + lx;
                    const int wt = m->wt[k];
                    if (sign > 0) {
                        if (wt == 0) {
                            m->sdf[k] = stored(m, sdf);
                            m->wt[k] = 1;
                        } else {
                            m->sdf[k] = stored(m, (m->sdf[k] * (real)wt + sdf) / (real)(wt + 1));
                            m->wt[k] = wt + 1 < m->max_w ? wt + 1 : m->max_w;
                        }
                    } else if (wt == 1) {
                        m->sdf[k] = 0;
                        m->wt[k] = 0;
                    } else if (wt > 1) {
                        m->sdf[k] = stored(m, (m->sdf[k] * (real)wt - sdf) / (real)(wt - 1));
                        m->wt[k] = wt - 1;
                    }
                }
    }
}

int orc_map_fuse(orc_map *m, const float *depth, int w, int h, const float *K, const double *Tcm) {
    orc_map_allocate(m, depth, w, h, K, Tcm);
    int *list = (int *)malloc(sizeof(int) * (m->n + 1));
    int n = collect_visible(m, w, h, K, Tcm, list);
    integrate(m, depth, w, h, K, Tcm, list, n, 1);
    free(list);
    return n;
}

int orc_map_defuse(orc_map *m, const float *depth, int w, int h, const float *K, const double *Tcm) {
    int *list = (int *)malloc(sizeof(int) * (m->n + 1));
    int n = collect_visible(m, w, h, K, Tcm, list);
    integrate(m, depth, w, h, K, Tcm, list, n, -1);
    free(list);
    return n;
}

void orc_map_export(const orc_map *m, int *coords, double *sdf, double *wt) {
    for (int i = 0; i < m->n; ++i) {
        if (coords) {
            coords[3 * i] = m->coords[3 * i];
            coords[3 * i + 1] = m->coords[3 * i + 1];
            coords[3 * i + 2] = m->coords[3 * i + 2];
        }
        for (int k = 0; k < 512; ++k) {
            if (sdf) sdf[(size_t)i * 512 + k] = (double)m->sdf[(size_t)i * 512 + k];
            if (wt) wt[(size_t)i * 512 + k] = (double)m->wt[(size_t)i * 512 + k];
        }
    }
}

void orc_map_import(orc_map *m, const int *coords, const float *sdf, const float *wt, int n) {
    for (int i = 0; i < n; ++i) {
        int b = insert_block(m, coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]);
        for (int k = 0; k < 512; ++k) {
            m->sdf[(size_t)b * 512 + k] = (real)sdf[(size_t)i * 512 + k];
            m->wt[(size_t)b * 512 + k] = (int)wt[(size_t)i * 512 + k];
        }
    }
}

/* ------------------------------------------------------------ submap fusion
 * MapStruct::Fuse(MapStruct*) (VoxelMap.cu:398-444): CreateBlockFunctor
 * (:231-262), then MapStructFusionFunctor (:363-396) with InterpolateSDF's
 * corner order and lerps (:305-361).  Poses: the maps' poses in the world
 * (3x4 row-major); source -> destination = inv(Tdst) Tsrc, composed in double
 * in the order of the library's host pose algebra and rounded once. */
static void pose_inv12(const double *T, double *o) {
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) o[i * 4 + j] = T[j * 4 + i];
        o[i * 4 + 3] = -((T[0 * 4 + i] * T[3] + T[1 * 4 + i] * T[7]) + T[2 * 4 + i] * T[11]);
    }
}

static void pose_mul12(const double *a, const double *b, double *o) {
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            o[i * 4 + j] = (a[i * 4 + 0] * b[0 * 4 + j] + a[i * 4 + 1] * b[1 * 4 + j]) + a[i * 4 + 2] * b[2 * 4 + j];
        o[i * 4 + 3] = ((a[i * 4 + 0] * b[3] + a[i * 4 + 1] * b[7]) + a[i * 4 + 2] * b[11]) + a[i * 4 + 3];
    }
}

static real read_voxel_w(const orc_map *m, int vx, int vy, int vz, int *wt) {
    int b = find_block(m, floor_div8(vx), floor_div8(vy), floor_div8(vz));
    if (b < 0) {
        *wt = 0;
        return 1;
    }
    const size_t k = (size_t)b * 512 + ((vz & 7) << 6) + ((vy & 7) << 3) + (vx & 7);
    *wt = m->wt[k];
    return *wt ? m->sdf[k] : 1;
}

static void map_clear(orc_map *m) {
    m->n = 0;
    for (int i = 0; i < m->hcap; ++i) m->hkey[i] = EMPTY_KEY;
}

/* Returns 1 when dst was empty and took src's storage (the caller swaps the
 * poses), else 0; src is left empty. */
int orc_map_fuse_map(orc_map *dst, orc_map *src, const double *Tdst, const double *Tsrc) {
    if (src->n == 0) return 0;
    if (dst->n == 0) {
        orc_map t = *dst;
        *dst = *src;
        *src = t;
        return 1;
    }
    double inv[12], t_sd[12], t_ds[12];
    pose_inv12(Tdst, inv);
    pose_mul12(inv, Tsrc, t_sd);
    pose_inv12(Tsrc, inv);
    pose_mul12(inv, Tdst, t_ds);
    const rig32 A = rig_from(t_sd), B = rig_from(t_ds);
    const float vs = dst->vs;
    for (int b = 0; b < src->n; ++b) {
        const int bx = src->coords[3 * b], by = src->coords[3 * b + 1], bz = src->coords[3 * b + 2];
        for (int li = 0; li < 512; ++li) {
            if (src->wt[(size_t)b * 512 + li] == 0) continue;
            float p[3];
            rig_apply(&A, (float)(bx * 8 + (li & 7)) * vs, (float)(by * 8 + ((li >> 3) & 7)) * vs,
                      (float)(bz * 8 + (li >> 6)) * vs, p);
            insert_block(dst, floor_div8(f2i_floor(p[0] / vs)), floor_div8(f2i_floor(p[1] / vs)),
                         floor_div8(f2i_floor(p[2] / vs)));
        }
    }
    const int ndst = dst->n;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int b = 0; b < ndst; ++b) {
        const int bx = dst->coords[3 * b], by = dst->coords[3 * b + 1], bz = dst->coords[3 * b + 2];
        for (int li = 0; li < 512; ++li) {
            float p[3];
            rig_apply(&B, (float)(bx * 8 + (li & 7)) * vs, (float)(by * 8 + ((li >> 3) & 7)) * vs,
                      (float)(bz * 8 + (li >> 6)) * vs, p);
            const float qx = p[0] / vs, qy = p[1] / vs, qz = p[2] / vs;
            const float fx = floorf(qx), fy = floorf(qy), fz = floorf(qz);
            const int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
            const real ax = (real)(qx - fx), ay = (real)(qy - fy), az = (real)(qz - fz);
            int w0, w;
            const real s000 = read_voxel_w(src, x0, y0, z0, &w0);
            if (!w0) continue;
            const real s100 = read_voxel_w(src, x0 + 1, y0, z0, &w);
            if (!w) continue;
            const real s010 = read_voxel_w(src, x0, y0 + 1, z0, &w);
            if (!w) continue;
            const real s110 = read_voxel_w(src, x0 + 1, y0 + 1, z0, &w);
            if (!w) continue;
            const real s001 = read_voxel_w(src, x0, y0, z0 + 1, &w);
            if (!w) continue;
            const real s101 = read_voxel_w(src, x0 + 1, y0, z0 + 1, &w);
            if (!w) continue;
            const real s011 = read_voxel_w(src, x0, y0 + 1, z0 + 1, &w);
            if (!w) continue;
            const real s111 = read_voxel_w(src, x0 + 1, y0 + 1, z0 + 1, &w);
            if (!w) continue;
            const real r0 = s000 * (1 - ax) + s100 * ax;
            const real r1 = r0 * (1 - ay) + (s010 * (1 - ax) + s110 * ax) * ay;
            const real r2 = s001 * (1 - ax) + s101 * ax;
            const real sv = r1 * (1 - az) + (r2 * (1 - ay) + (s011 * (1 - ax) + s111 * ax) * ay) * az;
            const size_t k = (size_t)b * 512 + li;
            const int dw = dst->wt[k];
            const real ds = dw ? dst->sdf[k] : 0;
            dst->sdf[k] = stored(dst, (ds * (real)dw + sv * (real)w0) / (real)(dw + w0));
            dst->wt[k] = dw + w0 < dst->max_w ? dw + w0 : dst->max_w;
        }
    }
    map_clear(src);
    return 0;
}

/* ------------------------------------------------------------ raycast */
static real read_voxel(const orc_map *m, int vx, int vy, int vz, int *valid) {
    int b = find_block(m, floor_div8(vx), floor_div8(vy), floor_div8(vz));
    if (b < 0) {
        *valid = 0;
        return 1;
    }
    const size_t k = (size_t)b * 512 + ((vz & 7) << 6) + ((vy & 7) << 3) + (vx & 7);
    if (m->wt[k] == 0) {
        *valid = 0;
        return 1;
    }
    *valid = 1;
    return m->sdf[k];
}

static real read_nearest(const orc_map *m, const real *p, int *valid) {
    return read_voxel(m, (int)floor(p[0]), (int)floor(p[1]), (int)floor(p[2]), valid);
}

/* Trilinear sample (RayTraceEngine.cu:346-378) over the cell floor(p) + {0,1}^3. */
static real read_interp(const orc_map *m, const real *p, int *valid) {
    const real fx = floor(p[0]), fy = floor(p[1]), fz = floor(p[2]);
    const int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
    const real ax = p[0] - fx, ay = p[1] - fy, az = p[2] - fz;
    int v0, v1, ok;
    real s0 = read_voxel(m, x0, y0, z0, &v0), s1 = read_voxel(m, x0 + 1, y0, z0, &v1);
    ok = v0 && v1;
    real r0 = (1 - ax) * s0 + ax * s1;
    s0 = read_voxel(m, x0, y0 + 1, z0, &v0);
    s1 = read_voxel(m, x0 + 1, y0 + 1, z0, &v1);
    ok = ok && v0 && v1;
    real r1 = (1 - ax) * s0 + ax * s1;
    const real r2 = (1 - ay) * r0 + ay * r1;
    s0 = read_voxel(m, x0, y0, z0 + 1, &v0);
    s1 = read_voxel(m, x0 + 1, y0, z0 + 1, &v1);
    ok = ok && v0 && v1;
    r0 = (1 - ax) * s0 + ax * s1;
    s0 = read_voxel(m, x0, y0 + 1, z0 + 1, &v0);
    s1 = read_voxel(m, x0 + 1, y0 + 1, z0 + 1, &v1);
    ok = ok && v0 && v1;
    r1 = (1 - ax) * s0 + ax * s1;
    const real r3 = (1 - ay) * r0 + ay * r1;
    *valid = ok;
    return (1 - az) * r2 + az * r3;
}

static int clamp_floor(float v) {
    if (!(v > -1.0e6f)) return -1000000;
    if (v > 1.0e6f) return 1000000;
    return (int)floorf(v);
}
static int clamp_ceil(float v) {
    if (!(v > -1.0e6f)) return -1000000;
    if (v > 1.0e6f) return 1000000;
    return (int)ceilf(v);
}

void orc_raycast(orc_map *m, int w, int h, const float *K, const double *Tcm, float *vmap, float *znear_out,
                 float *zfar_out) {
    const int zw = (w + 7) / 8, zh = (h + 7) / 8;
    float *zn = (float *)malloc(sizeof(float) * zw * zh), *zf = (float *)malloc(sizeof(float) * zw * zh);
    for (int i = 0; i < zw * zh; ++i) {
        zn[i] = 100.0f;
        zf[i] = 0.0f;
    }
    /* z-range of every visible block's footprint (RayTraceEngine.cu:124-174, 239-262) */
    int *list = (int *)malloc(sizeof(int) * (m->n + 1));
    const int nvis = collect_visible(m, w, h, K, Tcm, list);
    const rig32 Tinv = rig_inv_from(Tcm);
    const float scale = m->vs * 8.0f;
    for (int j = 0; j < nvis; ++j) {
        const int b = list[j];
        const int bx = m->coords[3 * b], by = m->coords[3 * b + 1], bz = m->coords[3 * b + 2];
        int ulx = zw, uly = zh, lrx = -1, lry = -1;
        float zmin = m->dmax, zmax = m->dmin;
        for (int c = 0; c < 8; ++c) {
            float p[3];
            rig_apply(&Tinv, (float)(bx + (c & 1)) * scale, (float)(by + ((c >> 1) & 1)) * scale,
                      (float)(bz + ((c >> 2) & 1)) * scale, p);
            const float u = ((K[0] * p[0]) / p[2] + K[2]) / 8.0f;
            const float v = ((K[1] * p[1]) / p[2] + K[3]) / 8.0f;
            int t;
            t = clamp_floor(u);
            if (t < ulx) ulx = t;
            t = clamp_floor(v);
            if (t < uly) uly = t;
            t = clamp_ceil(u);
            if (t > lrx) lrx = t;
            t = clamp_ceil(v);
            if (t > lry) lry = t;
            zmin = fminf(zmin, p[2]);
            zmax = fmaxf(zmax, p[2]);
        }
        if (ulx < 0) ulx = 0;
        if (uly < 0) uly = 0;
        if (lrx > zw - 1) lrx = zw - 1;
        if (lry > zh - 1) lry = zh - 1;
        if (ulx > lrx || uly > lry) continue;
        if (zmin < m->dmin) zmin = m->dmin;
        if (zmax < m->dmin) continue;
        for (int yy = uly; yy <= lry; ++yy)
            for (int xx = ulx; xx <= lrx; ++xx) {
                if (zmin < zn[yy * zw + xx]) zn[yy * zw + xx] = zmin;
                if (zmax > zf[yy * zw + xx]) zf[yy * zw + xx] = zmax;
            }
    }
    free(list);
    /* march (RayTraceEngine.cu:380-458) */
    const real vsinv = (real)1 / (real)m->vs;
    const real rstep = (real)m->trunc / (real)m->vs;
    const real invfx = (real)1 / (real)K[0], invfy = (real)1 / (real)K[1];
    const double *T = Tcm;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            float *out = vmap + ((size_t)y * w + x) * 4;
            out[0] = out[1] = out[2] = NAN;
            out[3] = -1.0f;
            const float znr = zn[(y >> 3) * zw + (x >> 3)], zfr = zf[(y >> 3) * zw + (x >> 3)];
            if (znr < FLT_EPSILON || zfr < FLT_EPSILON || isnan(znr) || isnan(zfr)) continue;
            const real ux = invfx * ((real)x - (real)K[2]), uy = invfy * ((real)y - (real)K[3]);
            real pn[3] = {ux * znr, uy * znr, (real)znr}, pf[3] = {ux * zfr, uy * zfr, (real)zfr};
            real dist_s = sqrt(pn[0] * pn[0] + pn[1] * pn[1] + pn[2] * pn[2]) * vsinv;
            const real dist_e = sqrt(pf[0] * pf[0] + pf[1] * pf[1] + pf[2] * pf[2]) * vsinv;
            real s[3], e[3];
            for (int i = 0; i < 3; ++i) {
                s[i] = (T[i * 4] * pn[0] + T[i * 4 + 1] * pn[1] + T[i * 4 + 2] * pn[2] + T[i * 4 + 3]) * vsinv;
                e[i] = (T[i * 4] * pf[0] + T[i * 4 + 1] * pf[1] + T[i * 4 + 2] * pf[2] + T[i * 4 + 3]) * vsinv;
            }
            real dir[3] = {e[0] - s[0], e[1] - s[1], e[2] - s[2]};
            const real dn = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
            if (dn > 0)
                for (int i = 0; i < 3; ++i) dir[i] /= dn;
            real r[3] = {s[0], s[1], s[2]};
            real sdf = 1;
            int valid = 0;
            while (dist_s < dist_e) {
                sdf = read_nearest(m, r, &valid);
                if (sdf <= 0.5 && sdf >= -0.5) sdf = read_interp(m, r, &valid);
                if (sdf <= 0) break;
                const real step = valid ? (sdf * rstep > 1 ? sdf * rstep : 1) : 1;
                for (int i = 0; i < 3; ++i) r[i] += step * dir[i];
                dist_s += step;
            }
            if (sdf <= 0) {
                real step = sdf * rstep;
                for (int i = 0; i < 3; ++i) r[i] += step * dir[i];
                sdf = read_interp(m, r, &valid);
                step = sdf * rstep;
                for (int i = 0; i < 3; ++i) r[i] += step * dir[i];
                if (valid) {
                    real wpt[3] = {r[0] / vsinv, r[1] / vsinv, r[2] / vsinv};
                    /* camera = R^T (w - t) */
                    for (int i = 0; i < 3; ++i)
                        out[i] = (float)(T[0 * 4 + i] * (wpt[0] - T[3]) + T[1 * 4 + i] * (wpt[1] - T[7]) +
                                         T[2 * 4 + i] * (wpt[2] - T[11]));
                    out[3] = 1.0f;
                }
            }
        }
    if (znear_out) memcpy(znear_out, zn, sizeof(float) * zw * zh);
    if (zfar_out) memcpy(zfar_out, zf, sizeof(float) * zw * zh);
    free(zn);
    free(zf);
}

/* ------------------------------------------------------------ marching cubes */
static const int CORNER[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const int EDGE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

/* Edge between corners a and b. */
static int edge_between(int a, int b) {
    for (int e = 0; e < 12; ++e)
        if ((EDGE[e][0] == a && EDGE[e][1] == b) || (EDGE[e][0] == b && EDGE[e][1] == a)) return e;
    return -1;
}

/*
 * Triangle table from cube topology.  For face f (axis f/2 at coordinate
 * f%2) the four corners are walked counter-clockwise about the outward
 * normal; a crossing edge is an "enter" when the walk steps onto an inside
 * (sdf < 0) corner and an "exit" otherwise.  Each exit is joined to the enter
 * that closes the inside region on its left: the only enter on a face with two
 * crossings, and on an ambiguous face (four crossings) the enter just before
 * it, which keeps the two inside corners apart.  The directed segments form
 * loops over the cube surface; each loop becomes a fan from its lowest edge.
 */
void orc_mc_tables(unsigned short *edge_out, signed char *tri_out, unsigned char *count_out) {
    for (int c = 0; c < 256; ++c) {
        unsigned short em = 0;
        for (int e = 0; e < 12; ++e)
            if (((c >> EDGE[e][0]) & 1) != ((c >> EDGE[e][1]) & 1)) em |= (unsigned short)(1u << e);
        if (edge_out) edge_out[c] = em;
        signed char *tri = tri_out ? tri_out + 31 * c : NULL;
        if (tri)
            for (int i = 0; i < 31; ++i) tri[i] = -1;
        int next[12];
        for (int e = 0; e < 12; ++e) next[e] = -1;
        for (int f = 0; f < 6; ++f) {
            const int axis = f / 2, side = f % 2, u = (axis + 1) % 3, v = (axis + 2) % 3;
            int ring[4] = {-1, -1, -1, -1};
            for (int k = 0; k < 8; ++k) {
                if (CORNER[k][axis] != side) continue;
                const int cu = CORNER[k][u], cv = CORNER[k][v];
                /* CCW about +axis: (0,0) (1,0) (1,1) (0,1) in (u, v) */
                const int pos = cv == 0 ? cu : 3 - cu;
                ring[pos] = k;
            }
            int q[4];
            if (side == 1) {
                for (int i = 0; i < 4; ++i) q[i] = ring[i];
            } else {
                q[0] = ring[0];
                q[1] = ring[3];
                q[2] = ring[2];
                q[3] = ring[1];
            }
            int ce[4], enter[4], nc = 0;
            for (int i = 0; i < 4; ++i) {
                const int a = q[i], b = q[(i + 1) & 3];
                const int ia = (c >> a) & 1, ib = (c >> b) & 1;
                if (ia != ib) {
                    ce[nc] = edge_between(a, b);
                    enter[nc] = ib;
                    ++nc;
                }
            }
            if (nc == 2) {
                if (enter[0])
                    next[ce[1]] = ce[0];
                else
                    next[ce[0]] = ce[1];
            } else if (nc == 4) {
                for (int i = 0; i < 4; ++i)
                    if (!enter[i]) next[ce[i]] = ce[(i + 3) & 3];
            }
        }
        int used[12] = {0}, ntri = 0, wpos = 0;
        for (int s = 0; s < 12; ++s) {
            if (!((em >> s) & 1) || used[s]) continue;
            int loop[12], k = 0, e = s;
            while (e >= 0 && !used[e] && k < 12) {
                used[e] = 1;
                loop[k++] = e;
                e = next[e];
            }
            for (int i = 1; i + 1 < k; ++i) {
                if (tri) {
                    tri[wpos++] = (signed char)loop[0];
                    tri[wpos++] = (signed char)loop[i];
                    tri[wpos++] = (signed char)loop[i + 1];
                }
                ++ntri;
            }
        }
        if (count_out) count_out[c] = (unsigned char)ntri;
    }
}

/* InterpolateSDF (MeshEngine.cu:140-149) */
static real mc_interp(real v1, real v2) {
    if (fabs(0 - v1) < 1e-6) return 0;
    if (fabs(0 - v2) < 1e-6) return 1;
    if (fabs(v1 - v2) < 1e-6) return 0;
    return (0 - v1) / (v2 - v1);
}

int orc_mesh(const orc_map *m, float *tris, float *normals, int *cases, int *cube_xyz, int cap) {
    static unsigned short edge[256];
    static signed char tri[256 * 31];
    static unsigned char cnt[256];
    static int ready = 0;
    if (!ready) {
        orc_mc_tables(edge, tri, cnt);
        ready = 1;
    }
    int ntri = 0;
    for (int b = 0; b < m->n; ++b) {
        const int bx = m->coords[3 * b], by = m->coords[3 * b + 1], bz = m->coords[3 * b + 2];
        for (int li = 0; li < 512; ++li) {
            const int gx = bx * 8 + (li & 7), gy = by * 8 + ((li >> 3) & 7), gz = bz * 8 + (li >> 6);
            real sd[8];
            int ok = 1, cidx = 0;
            for (int c = 0; c < 8 && ok; ++c) {
                int valid;
                sd[c] = read_voxel(m, gx + CORNER[c][0], gy + CORNER[c][1], gz + CORNER[c][2], &valid);
                if (!valid) ok = 0;
                else if (sd[c] < 0) cidx |= 1 << c;
            }
            if (!ok || cidx == 0 || edge[cidx] == 0) continue;
            real vt[12][3];
            const real px = gx, py = gy, pz = gz;
            for (int e = 0; e < 12; ++e) {
                if (!((edge[cidx] >> e) & 1)) continue;
                real *V = vt[e];
                switch (e) {
                    case 0: V[0] = px + mc_interp(sd[0], sd[1]); V[1] = py; V[2] = pz; break;
                    case 1: V[0] = px + 1; V[1] = py + mc_interp(sd[1], sd[2]); V[2] = pz; break;
                    case 2: V[0] = px + (1 - mc_interp(sd[2], sd[3])); V[1] = py + 1; V[2] = pz; break;
                    case 3: V[0] = px; V[1] = py + (1 - mc_interp(sd[3], sd[0])); V[2] = pz; break;
                    case 4: V[0] = px + mc_interp(sd[4], sd[5]); V[1] = py; V[2] = pz + 1; break;
                    case 5: V[0] = px + 1; V[1] = py + mc_interp(sd[5], sd[6]); V[2] = pz + 1; break;
                    case 6: V[0] = px + (1 - mc_interp(sd[6], sd[7])); V[1] = py + 1; V[2] = pz + 1; break;
                    case 7: V[0] = px; V[1] = py + (1 - mc_interp(sd[7], sd[4])); V[2] = pz + 1; break;
                    case 8: V[0] = px; V[1] = py; V[2] = pz + mc_interp(sd[0], sd[4]); break;
                    case 9: V[0] = px + 1; V[1] = py; V[2] = pz + mc_interp(sd[1], sd[5]); break;
                    case 10: V[0] = px + 1; V[1] = py + 1; V[2] = pz + mc_interp(sd[2], sd[6]); break;
                    default: V[0] = px; V[1] = py + 1; V[2] = pz + mc_interp(sd[3], sd[7]); break;
                }
            }
            for (int t = 0; t < cnt[cidx]; ++t, ++ntri) {
                if (ntri >= cap) continue;
                real v[3][3];
                for (int j = 0; j < 3; ++j)
                    for (int i = 0; i < 3; ++i) v[j][i] = vt[tri[31 * cidx + 3 * t + j]][i] * (real)m->vs;
                const real a[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
                const real c2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
                real n[3] = {a[1] * c2[2] - a[2] * c2[1], a[2] * c2[0] - a[0] * c2[2], a[0] * c2[1] - a[1] * c2[0]};
                const real nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                if (nn > 0)
                    for (int i = 0; i < 3; ++i) n[i] /= nn;
                for (int j = 0; j < 3; ++j)
                    for (int i = 0; i < 3; ++i) {
                        if (tris) tris[(size_t)ntri * 9 + 3 * j + i] = (float)v[j][i];
                        if (normals) normals[(size_t)ntri * 9 + 3 * j + i] = (float)n[i];
                    }
                if (cases) cases[ntri] = cidx;
                if (cube_xyz) {
                    cube_xyz[3 * ntri] = gx;
                    cube_xyz[3 * ntri + 1] = gy;
                    cube_xyz[3 * ntri + 2] = gz;
                }
            }
        }
    }
    return ntri;
}

int orc_real_bytes(void) { return (int)sizeof(real); }

/* ------------------------------------------------------------ shading
 * RenderScene (ImageProc.cu:80-139): Phong shading, white surface, ambient
 * 0.3, diffuse 0.5, specular 0.2 with power 20, point light in the camera
 * frame; a pixel without a vertex is (4, 2, 2, 255). */
static void normalise3(float *v) {
    const float n = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= n;
    v[1] /= n;
    v[2] /= n;
}

void orc_render_scene(const float *vmap, const float *nmap, int w, int h, const float *light, unsigned char *rgba) {
    for (int i = 0; i < w * h; ++i) {
        const float *p = vmap + 4 * (size_t)i, *nr = nmap + 4 * (size_t)i;
        unsigned char *o = rgba + 4 * (size_t)i;
        if (isnan(p[0])) {
            o[0] = 4;
            o[1] = 2;
            o[2] = 2;
            o[3] = 255;
            continue;
        }
        float L[3] = {light[0] - p[0], light[1] - p[1], light[2] - p[2]};
        float V[3] = {-p[0], -p[1], -p[2]};
        normalise3(L);
        normalise3(V);
        const float nl = nr[0] * L[0] + nr[1] * L[1] + nr[2] * L[2];
        float R[3] = {2.0f * nr[0] * nl - L[0], 2.0f * nr[1] * nl - L[1], 2.0f * nr[2] * nl - L[2]};
        normalise3(R);
        const float rv = R[0] * V[0] + R[1] * V[1] + R[2] * V[2];
        float I = 0.3f + 0.5f * fmaxf(0.0f, nl) + 0.2f * powf(fmaxf(0.0f, rv), 20.0f);
        I = I < 0.0f ? 0.0f : (I > 1.0f ? 1.0f : I);
        const unsigned char c = (unsigned char)(I * 255.0f);
        o[0] = o[1] = o[2] = c;
        o[3] = 255;
    }
}

/* ---------------------------------------------------------------- mesh canvas
 * MapDrawer's GLSL mesh program (FullSystem/src/MapDrawer.cpp:13-58, drawn by
 * :159-234) restated as a z-buffered rasteriser: per-vertex shading in the
 * submap frame, Tmw then Tcw, pinhole projection with pixel centres at
 * integer coordinates, perspective-correct interpolation, depth test on
 * (depth bits << 32 | RGBA).  Every operation is a single FP32 rounding in a
 * fixed order (this file is built without contraction). */
static float cv_dot(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

static void cv_normalize(float v[3]) {
    const float l = sqrtf(cv_dot(v, v));
    if (!(l > 0.0f)) {
        v[0] = v[1] = v[2] = 0.0f;
        return;
    }
    v[0] = v[0] / l;
    v[1] = v[1] / l;
    v[2] = v[2] / l;
}

static float cv_shade(const float p[3], const float n[3]) {
    float L[3] = {5.0f - p[0], 5.0f - p[1], 5.0f - p[2]};
    float V[3] = {-p[0], -p[1], -p[2]};
    cv_normalize(L);
    cv_normalize(V);
    const float nl = cv_dot(n, L);
    const float k = 2.0f * nl;
    float R[3] = {k * n[0] - L[0], k * n[1] - L[1], k * n[2] - L[2]};
    cv_normalize(R);
    const float rv = fmaxf(0.0f, cv_dot(R, V));
    const float r2 = rv * rv, r4 = r2 * r2, r8 = r4 * r4, r16 = r8 * r8, r20 = r16 * r4;
    const float i = (0.3f + 0.5f * fmaxf(0.0f, nl)) + 0.2f * r20;
    return fminf(1.0f, fmaxf(0.0f, i));
}

static void cv_apply(const float A[12], const float x[3], float o[3]) {
    for (int r = 0; r < 3; ++r) o[r] = ((A[r * 4] * x[0] + A[r * 4 + 1] * x[1]) + A[r * 4 + 2] * x[2]) + A[r * 4 + 3];
}

static float cv_edge(float ax, float ay, float bx, float by, float px, float py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

void orc_canvas_draw(const float *pts, const float *nrm, unsigned ntris, const double *Tmw, const double *Tcw,
                     const float *K4, int w, int h, uint64_t *keys) {
    float M[12], Vw[12];
    for (int i = 0; i < 12; ++i) {
        M[i] = (float)Tmw[i];
        Vw[i] = (float)Tcw[i];
    }
    const float fx = K4[0], fy = K4[1], cx = K4[2], cy = K4[3];
    for (unsigned t = 0; t < ntris; ++t) {
        float u[3], v[3], iz[3], ioz[3];
        int near = 0;
        for (int k = 0; k < 3; ++k) {
            const float *p = pts + (size_t)t * 9 + k * 3, *q = nrm + (size_t)t * 9 + k * 3;
            const float shade = cv_shade(p, q);
            float pw[3], pc[3];
            cv_apply(M, p, pw);
            cv_apply(Vw, pw, pc);
            near = near || !(pc[2] >= 0.05f);
            u[k] = (fx * pc[0]) / pc[2] + cx;
            v[k] = (fy * pc[1]) / pc[2] + cy;
            iz[k] = 1.0f / pc[2];
            ioz[k] = shade * iz[k];
        }
        if (near) continue;
        const float area = cv_edge(u[0], v[0], u[1], v[1], u[2], v[2]);
        if (!(area != 0.0f)) continue;
        const float lim = 1.0e7f;
        int x0 = (int)ceilf(fmaxf(-lim, fminf(fminf(u[0], u[1]), u[2])));
        int x1 = (int)floorf(fminf(lim, fmaxf(fmaxf(u[0], u[1]), u[2])));
        int y0 = (int)ceilf(fmaxf(-lim, fminf(fminf(v[0], v[1]), v[2])));
        int y1 = (int)floorf(fminf(lim, fmaxf(fmaxf(v[0], v[1]), v[2])));
        if (x0 < 0) x0 = 0;
        if (y0 < 0) y0 = 0;
        if (x1 > w - 1) x1 = w - 1;
        if (y1 > h - 1) y1 = h - 1;
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                const float px = (float)x, py = (float)y;
                const float e0 = cv_edge(u[1], v[1], u[2], v[2], px, py);
                const float e1 = cv_edge(u[2], v[2], u[0], v[0], px, py);
                const float e2 = cv_edge(u[0], v[0], u[1], v[1], px, py);
                const int in = area > 0.0f ? (e0 >= 0.0f && e1 >= 0.0f && e2 >= 0.0f)
                                           : (e0 <= 0.0f && e1 <= 0.0f && e2 <= 0.0f);
                if (!in) continue;
                const float b0 = e0 / area, b1 = e1 / area, b2 = e2 / area;
                const float wz = (b0 * iz[0] + b1 * iz[1]) + b2 * iz[2];
                if (!(wz > 0.0f)) continue;
                const float z = 1.0f / wz;
                const float wi = (b0 * ioz[0] + b1 * ioz[1]) + b2 * ioz[2];
                const float in01 = fminf(1.0f, fmaxf(0.0f, wi * z));
                const uint32_t c = (uint32_t)floorf(in01 * 255.0f + 0.5f);
                const uint32_t rgba = c | (c << 8) | (c << 16) | (255u << 24);
                uint32_t zb;
                memcpy(&zb, &z, 4);
                const uint64_t key = ((uint64_t)zb << 32) | rgba;
                uint64_t *dst = keys + (size_t)y * w + x;
                if (key < *dst) *dst = key;
            }
    }
}
