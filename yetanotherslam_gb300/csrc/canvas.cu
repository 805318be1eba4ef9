// canvas.cu — headless drawing of submap meshes into an RGBA image.
//
// The reference draws every inactive submap's marching-cubes mesh with a GLSL
// program (FullSystem/src/MapDrawer.cpp:13-58 shaders, :159-234 draw loop):
// the vertex shader shades each vertex in the submap's own frame with a
// light at (5, 5, 5) and the viewer at the origin,
//     I = 0.3 + 0.5 max(0, n.L) + 0.2 max(0, R.V)^20,
//     L = normalize(light - p), V = normalize(-p), R = normalize(2 n (n.L) - L),
// places it with mvpMat * Tmw, and OpenGL interpolates the colour over the
// triangle.  There is no GL here: a CUDA rasteriser restates it into a device
// buffer.  Each triangle is moved by Tmw (submap -> world) and Tcw (world ->
// camera), projected with pinhole intrinsics (pixel centres at integer
// coordinates), and every covered pixel takes the perspective-correct
// interpolated intensity.  The depth test is one 64-bit atomicMin per
// fragment on (depth bits << 32 | RGBA), so meshes drawn one after another
// share the z-buffer and equal depths resolve the same way in any order.
// Triangles with a vertex nearer than 5 cm are not drawn (no clipping).
// All arithmetic is one rounding per operation in a fixed order, so the image
// is reproducible bit for bit by a CPU restatement.
#include "yas_internal.h"

struct yas_canvas {
    int w = 0, h = 0;
    yas::Cam cam;
    cudaStream_t stream = nullptr;
    unsigned long long *keys = nullptr;  // w * h
};

namespace yas {

constexpr float kCanvasNear = 0.05f;
constexpr unsigned long long kCanvasEmpty = ~0ull;

struct Affine {
    float m[12];  // row-major [R | t]
};

__device__ __forceinline__ float3 affine_apply(const Affine &A, float x, float y, float z) {
    float3 o;
    o.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(A.m[0], x), __fmul_rn(A.m[1], y)), __fmul_rn(A.m[2], z)), A.m[3]);
    o.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(A.m[4], x), __fmul_rn(A.m[5], y)), __fmul_rn(A.m[6], z)), A.m[7]);
    o.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(A.m[8], x), __fmul_rn(A.m[9], y)), __fmul_rn(A.m[10], z)),
                    A.m[11]);
    return o;
}

__device__ __forceinline__ float dot3(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

__device__ __forceinline__ float3 normalize3(float3 v) {
    const float l = __fsqrt_rn(dot3(v, v));
    if (!(l > 0.0f)) return make_float3(0.0f, 0.0f, 0.0f);
    return make_float3(__fdiv_rn(v.x, l), __fdiv_rn(v.y, l), __fdiv_rn(v.z, l));
}

// The vertex shader's intensity (MapDrawer.cpp:26-44), in [0, 1].
__device__ __forceinline__ float mesh_shade(float3 p, float3 n) {
    const float3 L = normalize3(make_float3(__fsub_rn(5.0f, p.x), __fsub_rn(5.0f, p.y), __fsub_rn(5.0f, p.z)));
    const float3 V = normalize3(make_float3(-p.x, -p.y, -p.z));
    const float nl = dot3(n, L);
    const float k = __fmul_rn(2.0f, nl);
    const float3 R = normalize3(make_float3(__fsub_rn(__fmul_rn(k, n.x), L.x), __fsub_rn(__fmul_rn(k, n.y), L.y),
                                            __fsub_rn(__fmul_rn(k, n.z), L.z)));
    const float rv = fmaxf(0.0f, dot3(R, V));
    const float r2 = __fmul_rn(rv, rv), r4 = __fmul_rn(r2, r2), r8 = __fmul_rn(r4, r4), r16 = __fmul_rn(r8, r8);
    const float r20 = __fmul_rn(r16, r4);
    const float i = __fadd_rn(__fadd_rn(0.3f, __fmul_rn(0.5f, fmaxf(0.0f, nl))), __fmul_rn(0.2f, r20));
    return fminf(1.0f, fmaxf(0.0f, i));
}

// Twice the signed area of (a, b, p).
__device__ __forceinline__ float edge_fn(float ax, float ay, float bx, float by, float px, float py) {
    return __fsub_rn(__fmul_rn(__fsub_rn(bx, ax), __fsub_rn(py, ay)), __fmul_rn(__fsub_rn(by, ay), __fsub_rn(px, ax)));
}

__global__ void canvas_draw_kernel(const float *__restrict__ pts, const float *__restrict__ nrm, unsigned ntris,
                                   Affine model, Affine view, Cam cam, unsigned long long *keys, int w, int h) {
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < ntris; t += gridDim.x * blockDim.x) {
        float u[3], v[3], iz[3], ioz[3];
        bool near = false;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float *p = pts + (size_t)t * 9 + k * 3;
            const float *q = nrm + (size_t)t * 9 + k * 3;
            const float3 ps = make_float3(p[0], p[1], p[2]);
            const float shade = mesh_shade(ps, make_float3(q[0], q[1], q[2]));
            const float3 pw = affine_apply(model, ps.x, ps.y, ps.z);
            const float3 pc = affine_apply(view, pw.x, pw.y, pw.z);
            near = near || !(pc.z >= kCanvasNear);
            u[k] = __fadd_rn(__fdiv_rn(__fmul_rn(cam.fx, pc.x), pc.z), cam.cx);
            v[k] = __fadd_rn(__fdiv_rn(__fmul_rn(cam.fy, pc.y), pc.z), cam.cy);
            iz[k] = __fdiv_rn(1.0f, pc.z);
            ioz[k] = __fmul_rn(shade, iz[k]);
        }
        if (near) continue;
        const float area = edge_fn(u[0], v[0], u[1], v[1], u[2], v[2]);
        if (!(area != 0.0f)) continue;
        // bounds clamped before the conversion to int (a vertex at 5 cm can project far out)
        const float lim = 1.0e7f;
        const int x0 = max(0, (int)ceilf(fmaxf(-lim, fminf(fminf(u[0], u[1]), u[2]))));
        const int x1 = min(w - 1, (int)floorf(fminf(lim, fmaxf(fmaxf(u[0], u[1]), u[2]))));
        const int y0 = max(0, (int)ceilf(fmaxf(-lim, fminf(fminf(v[0], v[1]), v[2]))));
        const int y1 = min(h - 1, (int)floorf(fminf(lim, fmaxf(fmaxf(v[0], v[1]), v[2]))));
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                const float px = (float)x, py = (float)y;
                const float e0 = edge_fn(u[1], v[1], u[2], v[2], px, py);
                const float e1 = edge_fn(u[2], v[2], u[0], v[0], px, py);
                const float e2 = edge_fn(u[0], v[0], u[1], v[1], px, py);
                const bool in = area > 0.0f ? (e0 >= 0.0f && e1 >= 0.0f && e2 >= 0.0f)
                                            : (e0 <= 0.0f && e1 <= 0.0f && e2 <= 0.0f);
                if (!in) continue;
                const float b0 = __fdiv_rn(e0, area), b1 = __fdiv_rn(e1, area), b2 = __fdiv_rn(e2, area);
                const float wz = __fadd_rn(__fadd_rn(__fmul_rn(b0, iz[0]), __fmul_rn(b1, iz[1])), __fmul_rn(b2, iz[2]));
                if (!(wz > 0.0f)) continue;
                const float z = __fdiv_rn(1.0f, wz);
                const float wi = __fadd_rn(__fadd_rn(__fmul_rn(b0, ioz[0]), __fmul_rn(b1, ioz[1])), __fmul_rn(b2, ioz[2]));
                const float in01 = fminf(1.0f, fmaxf(0.0f, __fmul_rn(wi, z)));
                const unsigned c = (unsigned)floorf(__fadd_rn(__fmul_rn(in01, 255.0f), 0.5f));
                const unsigned rgba = c | (c << 8) | (c << 16) | (255u << 24);
                const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | rgba;
                atomicMin(keys + (size_t)y * w + x, key);
            }
    }
}

__global__ void canvas_resolve_kernel(const unsigned long long *keys, int w, int h, uchar4 *rgba, int rpitch,
                                      float *depth, int dpitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const unsigned long long k = keys[(size_t)y * w + x];
    const bool empty = k == kCanvasEmpty;
    if (rgba) {
        const unsigned c = empty ? 0xffffffffu : (unsigned)k;  // the viewer clears to white
        rgba[(size_t)y * rpitch + x] = make_uchar4(c & 255u, (c >> 8) & 255u, (c >> 16) & 255u, c >> 24);
    }
    if (depth) depth[(size_t)y * dpitch + x] = empty ? 0.0f : __uint_as_float((unsigned)(k >> 32));
}

static Affine affine_of(const yas_pose &p) {
    Affine a;
    for (int i = 0; i < 12; ++i) a.m[i] = (float)p.m[i];
    return a;
}

}  // namespace yas

using namespace yas;

extern "C" {

YAS_API int yas_canvas_destroy(yas_canvas *c) {
    if (!c) return YAS_ERR_BAD_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->keys);
    delete c;
    return YAS_OK;
}

YAS_API int yas_canvas_create(yas_canvas **out, int width, int height, const yas_intrinsics *K, void *stream) {
    if (!out || !K || width <= 0 || height <= 0 || width > 16384 || height > 16384) return YAS_ERR_BAD_ARG;
    yas_canvas *c = new yas_canvas();
    c->w = width;
    c->h = height;
    c->cam = make_cam(K->fx, K->fy, K->cx, K->cy, width, height);
    c->stream = (cudaStream_t)stream;
    if (cudaMalloc(&c->keys, (size_t)width * height * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return YAS_ERR_OOM;
    }
    *out = c;
    return yas_canvas_clear(c);
}

YAS_API int yas_canvas_clear(yas_canvas *c) {
    if (!c) return YAS_ERR_BAD_ARG;
    YAS_TRY_CUDA(cudaMemsetAsync(c->keys, 0xff, (size_t)c->w * c->h * sizeof(unsigned long long), c->stream));
    return YAS_OK;
}

YAS_API int yas_canvas_draw_triangles(yas_canvas *c, const float *points, const float *normals, unsigned n_tris,
                                      int on_device, const yas_pose *Tmw, const yas_pose *Tcw) {
    if (!c || !Tmw || !Tcw || (n_tris && (!points || !normals))) return YAS_ERR_BAD_ARG;
    if (!n_tris) return YAS_OK;
    const float *p = points, *n = normals;
    float *tmp = nullptr;
    if (!on_device) {
        const size_t bytes = (size_t)n_tris * 9 * sizeof(float);
        if (cudaMallocAsync(&tmp, 2 * bytes, c->stream) != cudaSuccess) {
            cudaGetLastError();
            return YAS_ERR_OOM;
        }
        YAS_TRY_CUDA(cudaMemcpyAsync(tmp, points, bytes, cudaMemcpyHostToDevice, c->stream));
        YAS_TRY_CUDA(cudaMemcpyAsync(tmp + (size_t)n_tris * 9, normals, bytes, cudaMemcpyHostToDevice, c->stream));
        p = tmp;
        n = tmp + (size_t)n_tris * 9;
    }
    const int grid = (int)std::min<unsigned>((n_tris + 127) / 128, (unsigned)kSMs * 16u);
    canvas_draw_kernel<<<grid, 128, 0, c->stream>>>(p, n, n_tris, affine_of(*Tmw), affine_of(*Tcw), c->cam, c->keys,
                                                    c->w, c->h);
    cudaError_t e = cudaGetLastError();
    if (tmp) {
        cudaFreeAsync(tmp, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    }
    YAS_TRY_CUDA(e);
    return YAS_OK;
}

YAS_API int yas_canvas_draw_mesh(yas_canvas *c, yas_mesher *me, const yas_pose *Tmw, const yas_pose *Tcw) {
    if (!c || !me) return YAS_ERR_BAD_ARG;
    const unsigned n = std::min<unsigned>(me->last_tris, (unsigned)me->mb.max_tris);
    if (me->stream != c->stream) YAS_TRY_CUDA(cudaStreamSynchronize(me->stream));
    return yas_canvas_draw_triangles(c, me->mb.points, me->mb.normals, n, 1, Tmw, Tcw);
}

YAS_API int yas_canvas_read(yas_canvas *c, uint8_t *rgba, int rgba_pitch, float *depth, int depth_pitch,
                            int on_device) {
    if (!c || (!rgba && !depth)) return YAS_ERR_BAD_ARG;
    if ((rgba && (rgba_pitch < c->w * 4 || rgba_pitch % 4)) || (depth && (depth_pitch < c->w * 4 || depth_pitch % 4)))
        return YAS_ERR_BAD_ARG;
    uchar4 *drgba = reinterpret_cast<uchar4 *>(rgba);
    float *ddepth = depth;
    void *tmp = nullptr;
    const size_t rb = (size_t)c->w * c->h * 4;
    if (!on_device) {
        if (cudaMallocAsync(&tmp, 2 * rb, c->stream) != cudaSuccess) {
            cudaGetLastError();
            return YAS_ERR_OOM;
        }
        drgba = rgba ? static_cast<uchar4 *>(tmp) : nullptr;
        ddepth = depth ? reinterpret_cast<float *>(static_cast<char *>(tmp) + rb) : nullptr;
    }
    const int rp = on_device ? rgba_pitch / 4 : c->w, dp = on_device ? depth_pitch / 4 : c->w;
    dim3 grid((c->w + 31) / 32, (c->h + 7) / 8);
    canvas_resolve_kernel<<<grid, dim3(32, 8), 0, c->stream>>>(c->keys, c->w, c->h, drgba, rp, ddepth, dp);
    cudaError_t e = cudaGetLastError();
    if (!on_device) {
        if (e == cudaSuccess && rgba)
            e = cudaMemcpy2DAsync(rgba, rgba_pitch, drgba, (size_t)c->w * 4, (size_t)c->w * 4, c->h,
                                  cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && depth)
            e = cudaMemcpy2DAsync(depth, depth_pitch, ddepth, (size_t)c->w * 4, (size_t)c->w * 4, c->h,
                                  cudaMemcpyDeviceToHost, c->stream);
        cudaFreeAsync(tmp, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    }
    YAS_TRY_CUDA(e);
    return YAS_OK;
}

}  // extern "C"
