// imgproc.cu — per-level image preprocessing for the dense tracker.
//
// Reference semantics (paths relative to the reference project root):
//   RGB -> gray            FullSystem/src/System.cpp:47-49 (cv::cvtColor RGB2GRAY): BT.601
//                          luma in 14-bit fixed point, gray = (4899 R + 9617 G + 1868 B
//                          + 8192) >> 14 (0.299/0.587/0.114 scaled by 2^14 and rounded).
//   u16 -> metres          System.cpp:52 (convertTo with the depth scale).
//   intensity pyramid      RGBDTracking.cu:66-116 (cv::cuda::pyrDown: separable
//                          [1 4 6 4 1]/16 Gaussian, reflect-101 border, keep even samples).
//   gradients              ImageProc.cu:7-40: 0.5 * central difference, 0 on the border.
//   inverse depth          ImageProc.cu:141-164: 1/z for 0.2 < z < 8, else 0.
//   nearest pyr-down       ImageProc.cu:166-187: dst(x,y) = src(2x,2y); the reference
//                          leaves the last row and column unwritten, here they are
//                          written as invalid (0 / w = -1).
//   vertex map             ImageProc.cu:189-220: z = 1/invz, valid when invz > 0 and z < 3.
//   normal map             ImageProc.cu:222-260: normalize((v(x,y+1)-v)x(v(x+1,y)-v)),
//                          invalid on the last row/column or when a vertex is invalid.
//   model pyramid          RGBDTracking.cu:140-150 (SetReferenceModel); the reference runs
//                          the float pyr-down on the float4 model (its coarse model levels
//                          are unusable); here the intended float4 nearest pyr-down is used.
#include <cstring>
#include <type_traits>

#include "yas_internal.h"
#include "yas_track.h"

namespace yas {

__device__ __forceinline__ float gray_of(const uint8_t *p, int channels, int bgr) {
    if (channels == 1) return (float)p[0];
    int r = bgr ? p[2] : p[0];
    int g = p[1];
    int b = bgr ? p[0] : p[2];
    return (float)((r * 4899 + g * 9617 + b * 1868 + 8192) >> 14);
}

// Level 0 intensity (+ gradients) from gray u8 or interleaved RGB u8.
__global__ void image_level0_kernel(const uint8_t *__restrict__ src, int channels, int bgr, int pitch,
                                    int w, int h, float *inten, float *gx, float *gy) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const uint8_t *row = src + (size_t)y * pitch;
    const float c = gray_of(row + x * channels, channels, bgr);
    inten[y * w + x] = c;
    if (x < 1 || y < 1 || x > w - 2 || y > h - 2) {
        gx[y * w + x] = 0.0f;
        gy[y * w + x] = 0.0f;
    } else {
        float l = gray_of(row + (x - 1) * channels, channels, bgr);
        float r = gray_of(row + (x + 1) * channels, channels, bgr);
        float u = gray_of(src + (size_t)(y - 1) * pitch + x * channels, channels, bgr);
        float d = gray_of(src + (size_t)(y + 1) * pitch + x * channels, channels, bgr);
        gx[y * w + x] = (r - l) * 0.5f;
        gy[y * w + x] = (d - u) * 0.5f;
    }
}

__device__ __forceinline__ int reflect101(int i, int n) {
    if (i < 0) i = -i;
    if (i >= n) i = 2 * (n - 1) - i;
    return i;
}

// Gaussian pyr-down of a float image: vertical 5-tap pass then horizontal.
__global__ void pyrdown_kernel(const float *__restrict__ src, int sw, int sh, float *dst, int dw, int dh) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    const float k[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
    int rows[5], cols[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        rows[i] = reflect101(2 * y + i - 2, sh);
        cols[i] = reflect101(2 * x + i - 2, sw);
    }
    // one rounding per operation, fixed order: the stored pyramid is bit-identical
    // to the CPU restatement's
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        float col = 0.0f;
#pragma unroll
        for (int i = 0; i < 5; ++i) col = __fadd_rn(col, __fmul_rn(k[i], __ldg(src + (size_t)rows[i] * sw + cols[j])));
        acc = __fadd_rn(acc, __fmul_rn(k[j], col));
    }
    dst[y * dw + x] = acc;
}

__global__ void gradient_kernel(const float *__restrict__ src, int w, int h, float *gx, float *gy) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    if (x < 1 || y < 1 || x > w - 2 || y > h - 2) {
        gx[y * w + x] = 0.0f;
        gy[y * w + x] = 0.0f;
    } else {
        gx[y * w + x] = (src[y * w + x + 1] - src[y * w + x - 1]) * 0.5f;
        gy[y * w + x] = (src[(y + 1) * w + x] - src[(y - 1) * w + x]) * 0.5f;
    }
}

__device__ __forceinline__ float inv_depth_of(float z) {
    return (z > 0.2f && z < 8.0f) ? 1.0f / z : 0.0f;
}

__device__ __forceinline__ float4 vertex_of(float invz, int x, int y, const LevelCam &c) {
    float z = 1.0f / invz;
    if (invz > 0.0f && z < 3.0f)
        return make_float4(z * ((float)x - c.cx) * c.invfx, z * ((float)y - c.cy) * c.invfy, z, 1.0f);
    return make_float4(0.0f, 0.0f, 0.0f, -1.0f);
}

__device__ __forceinline__ float4 normal_of(float4 v00, float4 v01, float4 v10) {
    if (v00.w > 0.0f && v01.w > 0.0f && v10.w > 0.0f) {
        // no contraction: normals (and so their validity and the ICP gates) are
        // bit-identical to the CPU restatement's
        float ax = v10.x - v00.x, ay = v10.y - v00.y, az = v10.z - v00.z;
        float bx = v01.x - v00.x, by = v01.y - v00.y, bz = v01.z - v00.z;
        float nx = __fsub_rn(__fmul_rn(ay, bz), __fmul_rn(az, by));
        float ny = __fsub_rn(__fmul_rn(az, bx), __fmul_rn(ax, bz));
        float nz = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
        float nn = __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
        if (nn > 0.0f) {
            float inv = 1.0f / sqrtf(nn);
            nx *= inv;
            ny *= inv;
            nz *= inv;
        }
        return make_float4(nx, ny, nz, 1.0f);
    }
    return make_float4(0.0f, 0.0f, 0.0f, -1.0f);
}

// Raw depth value at level 0 in metres (u16 * scale, or float).
__device__ __forceinline__ float raw_depth(const void *src, int is_u16, int pitch, float scale, int x, int y) {
    if (is_u16) return (float)reinterpret_cast<const uint16_t *>(static_cast<const char *>(src) + (size_t)y * pitch)[x] * scale;
    return reinterpret_cast<const float *>(static_cast<const char *>(src) + (size_t)y * pitch)[x];
}

// Depth of an inverse depth as the photometric warp uses it (1 / invd, one
// IEEE division), 0 where the inverse depth is invalid.
__device__ __forceinline__ float warp_depth_of(float invz) { return invz > 0.0f ? 1.0f / invz : 0.0f; }

// Level 0 depth: metres (optional), inverse depth, its reciprocal, vertex and
// normal maps.
__global__ void depth_level0_kernel(const void *__restrict__ src, int is_u16, int pitch, float scale,
                                    LevelCam c, float *depth_m, float *invd, float *zmap, float4 *vmap,
                                    float4 *nmap) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= c.w || y >= c.h) return;
    const float z = raw_depth(src, is_u16, pitch, scale, x, y);
    const float iz = inv_depth_of(z);
    if (depth_m) depth_m[y * c.w + x] = z;
    invd[y * c.w + x] = iz;
    zmap[y * c.w + x] = warp_depth_of(iz);
    const float4 v00 = vertex_of(iz, x, y, c);
    vmap[y * c.w + x] = v00;
    float4 n = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    if (x < c.w - 1 && y < c.h - 1) {
        float4 v01 = vertex_of(inv_depth_of(raw_depth(src, is_u16, pitch, scale, x + 1, y)), x + 1, y, c);
        float4 v10 = vertex_of(inv_depth_of(raw_depth(src, is_u16, pitch, scale, x, y + 1)), x, y + 1, c);
        n = normal_of(v00, v01, v10);
    }
    nmap[y * c.w + x] = n;
}

// Inverse depth of level l at (x,y) from level l-1 (nearest, last row/col invalid).
__device__ __forceinline__ float invd_down(const float *prev, int pw, int x, int y, int w, int h) {
    if (x >= w - 1 || y >= h - 1) return 0.0f;
    return __ldg(prev + (size_t)(2 * y) * pw + 2 * x);
}

__global__ void depth_pyr_kernel(const float *__restrict__ prev, int pw, LevelCam c, float *invd, float *zmap,
                                 float4 *vmap, float4 *nmap) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= c.w || y >= c.h) return;
    const float iz = invd_down(prev, pw, x, y, c.w, c.h);
    invd[y * c.w + x] = iz;
    zmap[y * c.w + x] = warp_depth_of(iz);
    const float4 v00 = vertex_of(iz, x, y, c);
    vmap[y * c.w + x] = v00;
    float4 n = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    if (x < c.w - 1 && y < c.h - 1) {
        float4 v01 = vertex_of(invd_down(prev, pw, x + 1, y, c.w, c.h), x + 1, y, c);
        float4 v10 = vertex_of(invd_down(prev, pw, x, y + 1, c.w, c.h), x, y + 1, c);
        n = normal_of(v00, v01, v10);
    }
    nmap[y * c.w + x] = n;
}

// The whole model pyramid in one launch (RGBDTracking.cu:140-150: level 0's
// normals, then each level's nearest pyr-down vertex map and its normals).
// Level l's vertex (x, y) of the chained pyr-down is level 0's vertex
// (2^l x, 2^l y) when x < w_l - 1 and y < h_l - 1 and invalid otherwise (the
// inner levels' conditions follow from the outer one), so every level reads
// the raycast's level-0 map directly and no level waits for another: the same
// values, one launch instead of one per level.  Thread i covers pixel i of the
// levels laid end to end.
struct ModelPyramid {
    int L, w[kMaxLevels], h[kMaxLevels], first[kMaxLevels + 1];
    float4 *vmap[kMaxLevels], *nmap[kMaxLevels];
};

__device__ __forceinline__ float4 model_vertex(const ModelPyramid &mp, int l, int x, int y) {
    if (l == 0) {
        if (x >= mp.w[0] || y >= mp.h[0]) return make_float4(0.0f, 0.0f, 0.0f, -1.0f);
        return mp.vmap[0][(size_t)y * mp.w[0] + x];
    }
    if (x >= mp.w[l] - 1 || y >= mp.h[l] - 1) return make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    return mp.vmap[0][(size_t)(y << l) * mp.w[0] + (x << l)];
}

__global__ void model_pyramid_kernel(const ModelPyramid mp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mp.first[mp.L]) return;
    int l = 0;
    while (l + 1 < mp.L && i >= mp.first[l + 1]) ++l;
    const int k = i - mp.first[l], w = mp.w[l], h = mp.h[l];
    const int y = k / w, x = k - y * w;
    const float4 v00 = model_vertex(mp, l, x, y);
    if (l > 0) mp.vmap[l][k] = v00;
    float4 n = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    if (x < w - 1 && y < h - 1) n = normal_of(v00, model_vertex(mp, l, x + 1, y), model_vertex(mp, l, x, y + 1));
    mp.nmap[l][k] = n;
}

void launch_model_pyramid(int L, const int *w, const int *h, float4 *const *vmap, float4 *const *nmap,
                          cudaStream_t s) {
    ModelPyramid mp;
    memset(&mp, 0, sizeof(mp));
    mp.L = L;
    mp.first[0] = 0;
    for (int l = 0; l < L; ++l) {
        mp.w[l] = w[l];
        mp.h[l] = h[l];
        mp.vmap[l] = vmap[l];
        mp.nmap[l] = nmap[l];
        mp.first[l + 1] = mp.first[l] + w[l] * h[l];
    }
    if (mp.first[L] == 0) return;
    model_pyramid_kernel<<<(mp.first[L] + 255) / 256, 256, 0, s>>>(mp);
}

static dim3 grid2(int w, int h) { return dim3((w + 31) / 32, (h + 7) / 8); }

void launch_image_level0(const uint8_t *src, int channels, int bgr, int pitch, int w, int h, float *inten,
                         float *gx, float *gy, cudaStream_t s) {
    image_level0_kernel<<<grid2(w, h), dim3(32, 8), 0, s>>>(src, channels, bgr, pitch, w, h, inten, gx, gy);
}

void launch_image_level(const float *prev, int pw, int ph, int w, int h, float *inten, float *gx, float *gy,
                        cudaStream_t s) {
    pyrdown_kernel<<<grid2(w, h), dim3(32, 8), 0, s>>>(prev, pw, ph, inten, w, h);
    if (gx) gradient_kernel<<<grid2(w, h), dim3(32, 8), 0, s>>>(inten, w, h, gx, gy);
}

void launch_depth_level0(const void *src, int is_u16, int pitch, float scale, const LevelCam &c,
                         float *depth_m, float *invd, float *zmap, float4 *vmap, float4 *nmap, cudaStream_t s) {
    depth_level0_kernel<<<grid2(c.w, c.h), dim3(32, 8), 0, s>>>(src, is_u16, pitch, scale, c, depth_m, invd,
                                                                 zmap, vmap, nmap);
}

void launch_depth_level(const float *prev, int pw, const LevelCam &c, float *invd, float *zmap, float4 *vmap,
                        float4 *nmap, cudaStream_t s) {
    depth_pyr_kernel<<<grid2(c.w, c.h), dim3(32, 8), 0, s>>>(prev, pw, c, invd, zmap, vmap, nmap);
}

// ---------------------------------------------------------------- shading
// RenderScene (ImageProc.cu:80-139): Phong shading of a vertex/normal map for
// display, white surface (ambient 0.3, diffuse 0.5, specular 0.2, power 20),
// point light at `light` (camera frame); a pixel without a vertex is
// (4, 2, 2, 255).  Colour bytes are the saturated intensity * 255 truncated.
__device__ __forceinline__ float3 normalised(float3 v) {
    const float n = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return make_float3(v.x / n, v.y / n, v.z / n);
}

__global__ void render_scene_kernel(const float4 *__restrict__ vmap, const float4 *__restrict__ nmap, int vpitch,
                                    int w, int h, float3 light, uchar4 *__restrict__ out, int opitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float4 p4 = vmap[(size_t)y * vpitch + x];
    const float4 n4 = nmap[(size_t)y * vpitch + x];
    uchar4 o = make_uchar4(4, 2, 2, 255);
    if (!isnan(p4.x)) {
        const float3 p = make_float3(p4.x, p4.y, p4.z), nrm = make_float3(n4.x, n4.y, n4.z);
        const float3 L = normalised(make_float3(light.x - p.x, light.y - p.y, light.z - p.z));
        const float3 V = normalised(make_float3(-p.x, -p.y, -p.z));
        const float nl = nrm.x * L.x + nrm.y * L.y + nrm.z * L.z;
        const float3 R = normalised(make_float3(2.0f * nrm.x * nl - L.x, 2.0f * nrm.y * nl - L.y, 2.0f * nrm.z * nl - L.z));
        const float rv = R.x * V.x + R.y * V.y + R.z * V.z;
        const float I = 0.3f + 0.5f * fmaxf(0.0f, nl) + 0.2f * powf(fmaxf(0.0f, rv), 20.0f);
        const unsigned char c = (unsigned char)(__saturatef(I) * 255.0f);
        o = make_uchar4(c, c, c, 255);
    }
    out[(size_t)y * opitch + x] = o;
}

void launch_render_scene(const float4 *vmap, const float4 *nmap, int vpitch, int w, int h, float3 light,
                         uchar4 *out, int opitch, cudaStream_t s) {
    dim3 block(32, 8);
    dim3 grid((w + 31) / 32, (h + 7) / 8);
    render_scene_kernel<<<grid, block, 0, s>>>(vmap, nmap, vpitch, w, h, light, out, opitch);
}

}  // namespace yas

// ---------------------------------------------------------------- free functions of ImageProc.h
// Standalone, pitched forms of the per-pixel functions the tracker fuses into
// its pyramid kernels, for callers of the reference's free functions
// (RGBDFusion/include/ImageProc.h:8-24).  One thread per pixel, 32x8 blocks.
namespace yas {

template <typename T>
__device__ __forceinline__ T *row_at(T *base, int pitch_bytes, int y) {
    return reinterpret_cast<T *>(reinterpret_cast<char *>(const_cast<typename std::remove_const<T>::type *>(base)) +
                                 (size_t)y * pitch_bytes);
}

__global__ void free_pyrdown_depth_kernel(const float *src, int spitch, float *dst, int dw, int dh, int dpitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    // PyrDownDepth_kernel: the last row and column are left as they are
    if (x >= dw - 1 || y >= dh - 1) return;
    row_at(dst, dpitch, y)[x] = row_at(src, spitch, 2 * y)[2 * x];
}

__global__ void free_inv_depth_kernel(const float *depth, int pitch, int w, int h, float *inv, int ipitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    row_at(inv, ipitch, y)[x] = inv_depth_of(row_at(depth, pitch, y)[x]);
}

__global__ void free_vertex_map_kernel(const float *invd, int pitch, int w, int h, float4 *vmap, int vpitch,
                                       float invfx, float invfy, float cx, float cy, float cut_off) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float invz = row_at(invd, pitch, y)[x];
    const float z = 1.0f / invz;
    float4 &o = row_at(vmap, vpitch, y)[x];
    if (invz > 0.0f && z < cut_off)
        o = make_float4(z * ((float)x - cx) * invfx, z * ((float)y - cy) * invfy, z, 1.0f);
    else
        o.w = -1.0f;  // ComputeVertexMap_kernel leaves x, y, z as they are
}

__global__ void free_normal_map_kernel(const float4 *vmap, int pitch, int w, int h, float4 *nmap, int npitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    float4 &o = row_at(nmap, npitch, y)[x];
    if (x == w - 1 || y == h - 1) {
        o.w = -1.0f;
        return;
    }
    const float4 n = normal_of(row_at(vmap, pitch, y)[x], row_at(vmap, pitch, y)[x + 1], row_at(vmap, pitch, y + 1)[x]);
    if (n.w > 0.0f)
        o = n;
    else
        o.w = -1.0f;
}

__global__ void free_gradient_kernel(const float *src, int pitch, int w, int h, float *gx, float *gy, int gpitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    float *ox = row_at(gx, gpitch, y) + x, *oy = row_at(gy, gpitch, y) + x;
    if (x < 1 || y < 1 || x > w - 2 || y > h - 2) {
        *ox = *oy = 0.0f;
    } else {
        const float *r = row_at(src, pitch, y);
        *ox = (r[x + 1] - r[x - 1]) * 0.5f;
        *oy = (row_at(src, pitch, y + 1)[x] - row_at(src, pitch, y - 1)[x]) * 0.5f;
    }
}

// TransformReferencePoint_kernel: RKinv (x, y, 1) z + t in FP32, Eigen's
// row-by-row product order, one rounding per operation.
__global__ void free_transform_points_kernel(const float *invd, int pitch, int w, int h, float4 *out, int opitch,
                                             Rigid32 RK) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float zinv = row_at(invd, pitch, y)[x];
    float4 &o = row_at(out, opitch, y)[x];
    if (zinv > 0.0f) {
        const float z = 1.0f / zinv, fx = (float)x, fy = (float)y;
        float p[3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
            p[i] = __fadd_rn(__fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(RK.r[i * 3], fx), __fmul_rn(RK.r[i * 3 + 1], fy)),
                                                 RK.r[i * 3 + 2]),
                                       z),
                             RK.t[i]);
        o = make_float4(p[0], p[1], p[2], 1.0f);
    } else {
        o = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    }
}

}  // namespace yas

using namespace yas;

namespace {
inline dim3 grid_of(int w, int h) { return dim3((unsigned)((w + 31) / 32), (unsigned)((h + 7) / 8)); }
inline bool bad_img(const void *p, int w, int h, int pitch, int elem) {
    return !p || w <= 0 || h <= 0 || pitch < w * elem || (pitch % elem) != 0;
}
}  // namespace

extern "C" {

YAS_API int yas_pyr_down_depth(const float *src, int src_w, int src_h, int src_pitch, float *dst, int dst_w,
                               int dst_h, int dst_pitch, void *stream) {
    if (bad_img(src, src_w, src_h, src_pitch, 4) || bad_img(dst, dst_w, dst_h, dst_pitch, 4) ||
        2 * (dst_w - 2) >= src_w || 2 * (dst_h - 2) >= src_h)
        return YAS_ERR_BAD_ARG;
    free_pyrdown_depth_kernel<<<grid_of(dst_w, dst_h), dim3(32, 8), 0, (cudaStream_t)stream>>>(
        src, src_pitch, dst, dst_w, dst_h, dst_pitch);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}

YAS_API int yas_depth_to_inv_depth(const float *depth, int w, int h, int pitch, float *inv_depth, int inv_pitch,
                                   void *stream) {
    if (bad_img(depth, w, h, pitch, 4) || bad_img(inv_depth, w, h, inv_pitch, 4)) return YAS_ERR_BAD_ARG;
    free_inv_depth_kernel<<<grid_of(w, h), dim3(32, 8), 0, (cudaStream_t)stream>>>(depth, pitch, w, h, inv_depth,
                                                                                   inv_pitch);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}

YAS_API int yas_compute_vertex_map(const float *inv_depth, int w, int h, int pitch, float *vmap, int vmap_pitch,
                                   float invfx, float invfy, float cx, float cy, float cut_off, void *stream) {
    if (bad_img(inv_depth, w, h, pitch, 4) || bad_img(vmap, w, h, vmap_pitch, 16)) return YAS_ERR_BAD_ARG;
    free_vertex_map_kernel<<<grid_of(w, h), dim3(32, 8), 0, (cudaStream_t)stream>>>(
        inv_depth, pitch, w, h, reinterpret_cast<float4 *>(vmap), vmap_pitch, invfx, invfy, cx, cy, cut_off);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}

YAS_API int yas_compute_normal_map(const float *vmap, int w, int h, int pitch, float *nmap, int nmap_pitch,
                                   void *stream) {
    if (bad_img(vmap, w, h, pitch, 16) || bad_img(nmap, w, h, nmap_pitch, 16)) return YAS_ERR_BAD_ARG;
    free_normal_map_kernel<<<grid_of(w, h), dim3(32, 8), 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(vmap), pitch, w, h, reinterpret_cast<float4 *>(nmap), nmap_pitch);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}

YAS_API int yas_image_gradient(const float *image, int w, int h, int pitch, float *gx, float *gy, int grad_pitch,
                               void *stream) {
    if (bad_img(image, w, h, pitch, 4) || bad_img(gx, w, h, grad_pitch, 4) || bad_img(gy, w, h, grad_pitch, 4))
        return YAS_ERR_BAD_ARG;
    free_gradient_kernel<<<grid_of(w, h), dim3(32, 8), 0, (cudaStream_t)stream>>>(image, pitch, w, h, gx, gy,
                                                                                  grad_pitch);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}

YAS_API int yas_transform_reference_point(const float *inv_depth, int w, int h, int pitch, float *vmap,
                                          int vmap_pitch, const double *K, const yas_pose *T, void *stream) {
    if (bad_img(inv_depth, w, h, pitch, 4) || bad_img(vmap, w, h, vmap_pitch, 16) || !K || !T) return YAS_ERR_BAD_ARG;
    // R * K^-1 in FP64, then rounded to FP32 (TransformReferencePoint, ImageProc.cu:64-78)
    const double fx = K[0], fy = K[4], cx = K[2], cy = K[5];
    if (!(fx != 0.0 && fy != 0.0)) return YAS_ERR_BAD_ARG;
    const double Ki[9] = {1.0 / fx, 0.0, -cx / fx, 0.0, 1.0 / fy, -cy / fy, 0.0, 0.0, 1.0};
    Rigid32 RK;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            RK.r[i * 3 + j] = (float)((T->m[i * 4 + 0] * Ki[0 * 3 + j] + T->m[i * 4 + 1] * Ki[1 * 3 + j]) +
                                      T->m[i * 4 + 2] * Ki[2 * 3 + j]);
        RK.t[i] = (float)T->m[i * 4 + 3];
    }
    free_transform_points_kernel<<<grid_of(w, h), dim3(32, 8), 0, (cudaStream_t)stream>>>(
        inv_depth, pitch, w, h, reinterpret_cast<float4 *>(vmap), vmap_pitch, RK);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}

YAS_API int yas_vmap_to_depth(const float *vmap, int w, int h, int pitch, float *depth, int depth_pitch,
                              void *stream) {
    if (bad_img(vmap, w, h, pitch, 16) || bad_img(depth, w, h, depth_pitch, 4)) return YAS_ERR_BAD_ARG;
    launch_vmap_to_depth(reinterpret_cast<const float4 *>(vmap), pitch / 16, depth, depth_pitch / 4, w, h,
                         (cudaStream_t)stream);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}

}  // extern "C"
