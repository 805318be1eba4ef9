// raycast.cu — TSDF raycasting into a camera-frame vertex map.
//
// Reference semantics (paths relative to the reference project root):
//   z-range tiles  RGBDFusion/src/RayTraceEngine.cu:58-214 (RenderingBlockDelegate,
//                  FillRenderingBlockFunctor): every visible block's 8 corners are
//                  projected to an (W/8)x(H/8) grid; each covered cell keeps the
//                  min near / max far depth of the blocks covering it.
//   ray march      RayTraceEngine.cu:266-410 (MapRenderingDelegate): march from the
//                  cell's near to far depth in voxel units with step
//                  max(sdf * trunc/voxel, 1) (1 when the sample is unobserved),
//                  trilinear sampling when |sdf| <= 0.5, stop at sdf <= 0, then two
//                  correction moves of sdf * trunc/voxel with one trilinear
//                  re-sample between them.
//
// GB300 design: the z-range fill walks each visible block's footprint with
// integer atomicMin/atomicMax on the float bit patterns (depths are positive,
// so integer order equals float order) instead of CAS loops over split tiles;
// the march caches the last block's pool index in registers, so consecutive
// samples inside one 8^3 block cost one 4- or 8-byte load each.
// Deliberate differences: a missed ray writes w = -1 (the reference leaves w
// stale on its early return, RayTraceEngine.cu:338-347); the 8 trilinear
// corners are floor(p) + {0,1}^3 (the reference floors p + offset per corner).
#include <algorithm>
#include <cfloat>

#include "yas_internal.h"

namespace yas {

__global__ void zrange_reset_kernel(float *znear, float *zfar, int n, unsigned *n_render, unsigned *queue,
                                    float *fnear, int nf) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        znear[i] = 100.0f;
        zfar[i] = 0.0f;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x) fnear[i] = 100.0f;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *n_render = 0;
        *queue = 0u;
    }
}

__device__ __forceinline__ int clamp_floor(float v) {
    if (!(v > -1.0e6f)) return -1000000;
    if (v > 1.0e6f) return 1000000;
    return (int)floorf(v);
}
__device__ __forceinline__ int clamp_ceil(float v) {
    if (!(v > -1.0e6f)) return -1000000;
    if (v > 1.0e6f) return 1000000;
    return (int)ceilf(v);
}

__global__ void __launch_bounds__(128) zrange_fill_kernel(MapDev m, Cam cam, const PosePair *P,
                                                          float *znear, float *zfar, int zw, int zh,
                                                          const int *skip, float *fnear, int fw, int fh) {
    if (skip && *skip) return;
    const unsigned nvis = *(volatile unsigned *)&m.hdr->n_visible;
    const Rigid32 Tinv = P->Tinv;
    const float scale = m.voxel_size * 8.0f;
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < nvis; j += gridDim.x * blockDim.x) {
        int bx, by, bz;
        unpack_key(m.block_keys[m.visible[j]], bx, by, bz);
        int ulx = zw, uly = zh, lrx = -1, lry = -1;
        float zmin = m.depth_max, zmax = m.depth_min;
        float pu0 = 1e30f, pu1 = -1e30f, pv0 = 1e30f, pv1 = -1e30f;
        bool behind = false;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            float3 p = rigid_exact(Tinv, (float)(bx + (c & 1)) * scale, (float)(by + ((c >> 1) & 1)) * scale,
                                   (float)(bz + ((c >> 2) & 1)) * scale);
            const float pu = cam.fx * p.x / p.z + cam.cx, pv = cam.fy * p.y / p.z + cam.cy;
            float u = pu / 8.0f;
            float v = pv / 8.0f;
            ulx = min(ulx, clamp_floor(u));
            uly = min(uly, clamp_floor(v));
            lrx = max(lrx, clamp_ceil(u));
            lry = max(lry, clamp_ceil(v));
            zmin = fminf(zmin, p.z);
            zmax = fmaxf(zmax, p.z);
            behind = behind || !(p.z > 1e-3f);
            pu0 = fminf(pu0, pu);
            pu1 = fmaxf(pu1, pu);
            pv0 = fminf(pv0, pv);
            pv1 = fmaxf(pv1, pv);
        }
        // Fine near bound (not a reference quantity; the march uses it only to
        // jump over samples that lie before every visible block along the ray):
        // the block's projected box widened by a pixel, or the whole image when a
        // corner is not in front of the camera.
        if (zmax >= m.depth_min) {
            int fx0 = 0, fy0 = 0, fx1 = fw - 1, fy1 = fh - 1;
            if (!behind) {
                constexpr float kInvCell = 1.0f / (float)(1 << kFineShift);
                fx0 = max(fx0, clamp_floor((pu0 - 1.0f) * kInvCell));
                fy0 = max(fy0, clamp_floor((pv0 - 1.0f) * kInvCell));
                fx1 = min(fx1, clamp_floor((pu1 + 1.0f) * kInvCell));
                fy1 = min(fy1, clamp_floor((pv1 + 1.0f) * kInvCell));
            }
            const int fz = __float_as_int(fmaxf(fminf(zmin, m.depth_max), 0.0f));
            for (int y = fy0; y <= fy1; ++y)
                for (int x = fx0; x <= fx1; ++x) atomicMin(reinterpret_cast<int *>(fnear) + y * fw + x, fz);
        }
        ulx = max(ulx, 0);
        uly = max(uly, 0);
        lrx = min(lrx, zw - 1);
        lry = min(lry, zh - 1);
        if (ulx > lrx || uly > lry) continue;
        if (zmin < m.depth_min) zmin = m.depth_min;
        if (zmax < m.depth_min) continue;
        const int inear = __float_as_int(zmin), ifar = __float_as_int(zmax);
        for (int y = uly; y <= lry; ++y)
            for (int x = ulx; x <= lrx; ++x) {
                atomicMin(reinterpret_cast<int *>(znear) + y * zw + x, inear);
                atomicMax(reinterpret_cast<int *>(zfar) + y * zw + x, ifar);
            }
        unsigned tiles = (unsigned)(((lrx - ulx + 16) / 16) * ((lry - uly + 16) / 16));
        atomicAdd(&m.hdr->n_render, tiles);
    }
}

void launch_zrange(const MapDev &m, const Cam &cam, const PosePair *P, RaycastBuffers &rb,
                   const int *skip, cudaStream_t s) {
    const int n = rb.zw * rb.zh, nf = rb.fw * rb.fh;
    zrange_reset_kernel<<<(std::max(n, nf) + 255) / 256, 256, 0, s>>>(rb.znear, rb.zfar, n, &m.hdr->n_render,
                                                                      rb.queue, rb.fnear, nf);
    zrange_fill_kernel<<<kSMs * 2, 128, 0, s>>>(m, cam, P, rb.znear, rb.zfar, rb.zw, rb.zh, skip, rb.fnear, rb.fw,
                                               rb.fh);
}

// Block-pointer cache of one ray.
template <int FMT>
struct VoxelReader {
    typedef VoxelIO<FMT> IO;
    const MapDev &m;
    const typename IO::T *vox;
    unsigned long long ckey;
    int cptr;
    __device__ __forceinline__ VoxelReader(const MapDev &mm)
        : m(mm), vox(static_cast<const typename IO::T *>(mm.voxels)), ckey(kEmptyKey), cptr(-1) {}

    // sdf of voxel (vx,vy,vz); valid = observed (weight != 0)
    __device__ __forceinline__ float read(int vx, int vy, int vz, bool &valid) {
        int bx = vx >> 3, by = vy >> 3, bz = vz >> 3;
        unsigned long long k = pack_key(bx, by, bz);
        if (k != ckey) {
            ckey = k;
            cptr = coord_in_range(bx, by, bz) ? find_block(m, k) : -1;
        }
        if (cptr < 0) {
            valid = false;
            return 1.0f;
        }
        typename IO::T v = __ldg(vox + (size_t)cptr * kBlockVoxels + ((vz & 7) << 6) + ((vy & 7) << 3) + (vx & 7));
        if (IO::wt(v) == 0) {
            valid = false;
            return 1.0f;
        }
        valid = true;
        return IO::sdf(v);
    }
    __device__ __forceinline__ float read_nearest(float3 p, bool &valid) {
        return read((int)floorf(p.x), (int)floorf(p.y), (int)floorf(p.z), valid);
    }
    // Trilinear sample with the reference's lerp order (RayTraceEngine.cu:297-329).
    __device__ __forceinline__ float corner(typename IO::T v, bool &ok) {
        if (IO::wt(v) == 0) {
            ok = false;
            return 1.0f;
        }
        return IO::sdf(v);
    }
    __device__ __forceinline__ float read_interp(float3 p, bool &valid) {
        float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
        int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
        float ax = p.x - fx, ay = p.y - fy, az = p.z - fz;
        if ((x0 & 7) != 7 && (y0 & 7) != 7 && (z0 & 7) != 7) {
            // the 2x2x2 cell lies in one block: eight independent loads at
            // fixed offsets from one base, same lerp order as the general path
            int bx = x0 >> 3, by = y0 >> 3, bz = z0 >> 3;
            unsigned long long k = pack_key(bx, by, bz);
            if (k != ckey) {
                ckey = k;
                cptr = coord_in_range(bx, by, bz) ? find_block(m, k) : -1;
            }
            if (cptr < 0) {
                valid = false;
                return 1.0f;
            }
            const typename IO::T *b =
                vox + (size_t)cptr * kBlockVoxels + ((z0 & 7) << 6) + ((y0 & 7) << 3) + (x0 & 7);
            const typename IO::T q0 = __ldg(b), q1 = __ldg(b + 1), q2 = __ldg(b + 8), q3 = __ldg(b + 9);
            const typename IO::T q4 = __ldg(b + 64), q5 = __ldg(b + 65), q6 = __ldg(b + 72), q7 = __ldg(b + 73);
            bool ok = true;
            const float s000 = corner(q0, ok), s100 = corner(q1, ok), s010 = corner(q2, ok), s110 = corner(q3, ok);
            const float s001 = corner(q4, ok), s101 = corner(q5, ok), s011 = corner(q6, ok), s111 = corner(q7, ok);
            float r0 = (1.0f - ax) * s000 + ax * s100;
            float r1 = (1.0f - ax) * s010 + ax * s110;
            const float r2 = (1.0f - ay) * r0 + ay * r1;
            r0 = (1.0f - ax) * s001 + ax * s101;
            r1 = (1.0f - ax) * s011 + ax * s111;
            const float r3 = (1.0f - ay) * r0 + ay * r1;
            valid = ok;
            return (1.0f - az) * r2 + az * r3;
        }
        bool v0, v1, ok = true;
        float s0 = read(x0, y0, z0, v0);
        float s1 = read(x0 + 1, y0, z0, v1);
        ok = v0 && v1;
        float r0 = (1.0f - ax) * s0 + ax * s1;
        s0 = read(x0, y0 + 1, z0, v0);
        s1 = read(x0 + 1, y0 + 1, z0, v1);
        ok = ok && v0 && v1;
        float r1 = (1.0f - ax) * s0 + ax * s1;
        float r2 = (1.0f - ay) * r0 + ay * r1;
        s0 = read(x0, y0, z0 + 1, v0);
        s1 = read(x0 + 1, y0, z0 + 1, v1);
        ok = ok && v0 && v1;
        r0 = (1.0f - ax) * s0 + ax * s1;
        s0 = read(x0, y0 + 1, z0 + 1, v0);
        s1 = read(x0 + 1, y0 + 1, z0 + 1, v1);
        ok = ok && v0 && v1;
        r1 = (1.0f - ax) * s0 + ax * s1;
        float r3 = (1.0f - ay) * r0 + ay * r1;
        valid = ok;
        return (1.0f - az) * r2 + az * r3;
    }
};

// State of one ray of the march (RayTraceEngine.cu:331-410), in voxel units.
struct RayState {
    float3 r, dir, idir;
    float dist_s, dist_e, sdf;
    bool valid;
    unsigned long long skipped;
};

// Ray of pixel (x, y) between the tile's z-range bounds zn..zf; false when the
// tile has no range (the pixel is a miss).  zfine: the nearest visible block
// whose projected box covers the pixel's 4x4 neighbourhood.  The march starts
// at zn as the reference's does; every sample before zfine lies outside every
// visible block, reads "unobserved" and advances one voxel, so those samples
// are taken in one move (two are kept as margin against rounding).
__device__ __forceinline__ bool ray_setup(const Cam &cam, const Rigid32 &T, float vsinv, float zn, float zf,
                                          float zfine, int x, int y, RayState &R) {
    if (zn < FLT_EPSILON || zf < FLT_EPSILON || isnan(zn) || isnan(zf)) return false;
    const float ux = cam.invfx * ((float)x - cam.cx), uy = cam.invfy * ((float)y - cam.cy);
    const float3 pn = make_float3(ux * zn, uy * zn, zn);
    R.dist_s = sqrtf(pn.x * pn.x + pn.y * pn.y + pn.z * pn.z) * vsinv;
    float3 s = rigid_fast(T, pn.x, pn.y, pn.z);
    s = make_float3(s.x * vsinv, s.y * vsinv, s.z * vsinv);
    const float3 pf = make_float3(ux * zf, uy * zf, zf);
    R.dist_e = sqrtf(pf.x * pf.x + pf.y * pf.y + pf.z * pf.z) * vsinv;
    float3 e = rigid_fast(T, pf.x, pf.y, pf.z);
    e = make_float3(e.x * vsinv, e.y * vsinv, e.z * vsinv);
    float3 dir = make_float3(e.x - s.x, e.y - s.y, e.z - s.z);
    const float dn = sqrtf(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
    if (dn > 0.0f) dir = make_float3(dir.x / dn, dir.y / dn, dir.z / dn);
    R.r = s;
    R.dir = dir;
    R.idir = make_float3(dir.x != 0.0f ? 1.0f / dir.x : 0.0f, dir.y != 0.0f ? 1.0f / dir.y : 0.0f,
                         dir.z != 0.0f ? 1.0f / dir.z : 0.0f);
    R.skipped = kEmptyKey;
    R.sdf = 1.0f;
    R.valid = false;
    if (zfine > zn) {
        const float k = sqrtf(ux * ux + uy * uy + 1.0f) * vsinv;  // voxels of ray per metre of depth
        const float n = floorf(fminf(zfine * k, R.dist_e) - R.dist_s) - 2.0f;
        if (n >= 1.0f) {
            R.r = make_float3(R.r.x + n * dir.x, R.r.y + n * dir.y, R.r.z + n * dir.z);
            R.dist_s += n;
        }
    }
    return true;
}

// One iteration of the march loop; true once the ray is finished (a sample
// with sdf <= 0, or the end of its range).
template <int FMT>
__device__ __forceinline__ bool ray_step(VoxelReader<FMT> &rd, float rstep, RayState &R) {
    if (!(R.dist_s < R.dist_e)) return true;
    R.sdf = rd.read_nearest(R.r, R.valid);
    if (rd.cptr < 0 && rd.ckey != R.skipped) {
        // Unallocated block: every sample until the ray leaves it reads
        // "unobserved" and advances one voxel, so those samples are skipped in
        // one move.  k = steps to the first sample outside the block on the
        // earliest exit axis.  When sample k - 1 (computed as the jump computes
        // it) is still in the block and sample k is not, the ray jumps straight
        // to sample k; otherwise (k rounded the wrong way) it keeps two samples
        // as margin and evaluates the last ones inside the block normally.
        R.skipped = rd.ckey;
        const float bx0 = floorf(floorf(R.r.x) * 0.125f) * 8.0f;
        const float by0 = floorf(floorf(R.r.y) * 0.125f) * 8.0f;
        const float bz0 = floorf(floorf(R.r.z) * 0.125f) * 8.0f;
        const float kx = R.dir.x > 0.0f ? ceilf((bx0 + 8.0f - R.r.x) * R.idir.x)
                                        : (R.dir.x < 0.0f ? floorf((bx0 - R.r.x) * R.idir.x) + 1.0f : 1e30f);
        const float ky = R.dir.y > 0.0f ? ceilf((by0 + 8.0f - R.r.y) * R.idir.y)
                                        : (R.dir.y < 0.0f ? floorf((by0 - R.r.y) * R.idir.y) + 1.0f : 1e30f);
        const float kz = R.dir.z > 0.0f ? ceilf((bz0 + 8.0f - R.r.z) * R.idir.z)
                                        : (R.dir.z < 0.0f ? floorf((bz0 - R.r.z) * R.idir.z) + 1.0f : 1e30f);
        const float k = fminf(fminf(kx, ky), kz);
        float n = k - 2.0f;
        if (k >= 1.0f && k < 1e29f) {
            const float a = k - 1.0f;
            const float3 pin = make_float3(R.r.x + a * R.dir.x, R.r.y + a * R.dir.y, R.r.z + a * R.dir.z);
            const float3 pout = make_float3(R.r.x + k * R.dir.x, R.r.y + k * R.dir.y, R.r.z + k * R.dir.z);
            const unsigned long long kin =
                pack_key((int)floorf(pin.x) >> 3, (int)floorf(pin.y) >> 3, (int)floorf(pin.z) >> 3);
            const unsigned long long kout =
                pack_key((int)floorf(pout.x) >> 3, (int)floorf(pout.y) >> 3, (int)floorf(pout.z) >> 3);
            if (kin == rd.ckey && kout != rd.ckey) n = k;
        }
        n = fminf(n, ceilf(R.dist_e - R.dist_s));
        if (n >= 1.0f) {
            R.r.x += n * R.dir.x;
            R.r.y += n * R.dir.y;
            R.r.z += n * R.dir.z;
            R.dist_s += n;
            return false;
        }
    }
    if (R.sdf <= 0.5f && R.sdf >= -0.5f) R.sdf = rd.read_interp(R.r, R.valid);
    if (R.sdf <= 0.0f) return true;
    const float step = R.valid ? fmaxf(R.sdf * rstep, 1.0f) : 1.0f;
    R.r.x += step * R.dir.x;
    R.r.y += step * R.dir.y;
    R.r.z += step * R.dir.z;
    R.dist_s += step;
    return false;
}

// Vertex of a finished ray: a hit takes two interpolated correction steps
// and is returned in camera coordinates (w = 1); a miss is NaN with w = -1.
template <int FMT>
__device__ __forceinline__ float4 ray_finish(VoxelReader<FMT> &rd, float rstep, float vsinv, const Rigid32 &Ti,
                                             RayState &R) {
    float4 out = make_float4(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff), __int_as_float(0x7fffffff),
                             -1.0f);
    if (R.sdf <= 0.0f) {
        float step = R.sdf * rstep;
        R.r.x += step * R.dir.x;
        R.r.y += step * R.dir.y;
        R.r.z += step * R.dir.z;
        R.sdf = rd.read_interp(R.r, R.valid);
        step = R.sdf * rstep;
        R.r.x += step * R.dir.x;
        R.r.y += step * R.dir.y;
        R.r.z += step * R.dir.z;
        if (R.valid) {
            const float3 w = make_float3(R.r.x / vsinv, R.r.y / vsinv, R.r.z / vsinv);
            const float3 c = rigid_fast(Ti, w.x, w.y, w.z);
            out = make_float4(c.x, c.y, c.z, 1.0f);
        }
    }
    return out;
}

// One thread per pixel; each warp a compact 8x4 tile, so its rays travel
// similar depths; the CTA's WX x WY warp tiles cover 8WX x 4WY pixels.
template <int FMT, int WX, int WY>
__global__ void __launch_bounds__(32 * WX * WY) march_kernel(MapDev m, Cam cam, const PosePair *P,
                                                             const float *__restrict__ znear,
                                                             const float *__restrict__ zfar, int zw, float4 *vmap,
                                                             int vpitch, const int *skip,
                                                             const float *__restrict__ fnear, int fw) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x = blockIdx.x * (8 * WX) + (warp % WX) * 8 + (lane & 7);
    const int y = blockIdx.y * (4 * WY) + (warp / WX) * 4 + (lane >> 3);
    if (x >= cam.w || y >= cam.h) return;
    float4 out = make_float4(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff), __int_as_float(0x7fffffff),
                             -1.0f);
    if (!(skip && *skip)) {
        const float vsinv = 1.0f / m.voxel_size;
        const float rstep = m.trunc / m.voxel_size;
        RayState R;
        if (ray_setup(cam, P->T, vsinv, __ldg(znear + (y >> 3) * zw + (x >> 3)), __ldg(zfar + (y >> 3) * zw + (x >> 3)),
                      __ldg(fnear + (y >> kFineShift) * fw + (x >> kFineShift)), x, y, R)) {
            VoxelReader<FMT> rd(m);
            while (!ray_step(rd, rstep, R)) {
            }
            out = ray_finish(rd, rstep, vsinv, P->Tinv, R);
        }
    }
    vmap[(size_t)y * vpitch + x] = out;
}

// Persistent march: resident warps take 8x4-pixel tiles from a queue (one
// atomic per tile on rb.queue, tiles row-major), a warp taking the next tile
// once all its rays are done, so no SM idles behind a partial last wave.
// Each ray runs exactly the steps of march_kernel, so the vertex map is the
// same bit for bit.
template <int FMT>
__global__ void __launch_bounds__(128) march_persistent_kernel(MapDev m, Cam cam, const PosePair *P,
                                                               const float *__restrict__ znear,
                                                               const float *__restrict__ zfar, int zw, float4 *vmap,
                                                               int vpitch, const int *skip, unsigned *queue,
                                                               unsigned total, const float *__restrict__ fnear,
                                                               int fw) {
    const unsigned lane = lane_id();
    const int tiles_x = (cam.w + 7) >> 3;
    const float4 miss = make_float4(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff),
                                    __int_as_float(0x7fffffff), -1.0f);
    if (skip && *skip) {
        for (unsigned p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
            const int t = (int)(p >> 5), l = (int)(p & 31u);
            const int x = (t % tiles_x) * 8 + (l & 7), y = (t / tiles_x) * 4 + (l >> 3);
            if (x < cam.w && y < cam.h) vmap[(size_t)y * vpitch + x] = miss;
        }
        return;
    }
    const float vsinv = 1.0f / m.voxel_size;
    const float rstep = m.trunc / m.voxel_size;
    VoxelReader<FMT> rd(m);
    RayState R;
    bool active = false, drained = false;
    int x = 0, y = 0;
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active);
        if (!drained && idle == 0xffffffffu) {
            const int leader = __ffs(idle) - 1;
            unsigned base = 0u;
            if ((int)lane == leader) base = atomicAdd(queue, (unsigned)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + (unsigned)__popc(idle) >= total) drained = true;
            if (!active) {
                const unsigned p = base + (unsigned)__popc(idle & ((1u << lane) - 1u));
                if (p < total) {
                    const int t = (int)(p >> 5), l = (int)(p & 31u);
                    x = (t % tiles_x) * 8 + (l & 7);
                    y = (t / tiles_x) * 4 + (l >> 3);
                    if (x < cam.w && y < cam.h) {
                        if (ray_setup(cam, P->T, vsinv, __ldg(znear + (y >> 3) * zw + (x >> 3)),
                                      __ldg(zfar + (y >> 3) * zw + (x >> 3)), __ldg(fnear + (y >> kFineShift) * fw + (x >> kFineShift)),
                                      x, y, R))
                            active = true;
                        else
                            vmap[(size_t)y * vpitch + x] = miss;
                    }
                }
            }
        }
        if (__ballot_sync(0xffffffffu, active) == 0u) {
            if (drained) break;
            continue;
        }
        if (active && ray_step(rd, rstep, R)) {
            vmap[(size_t)y * vpitch + x] = ray_finish(rd, rstep, vsinv, P->Tinv, R);
            active = false;
        }
    }
}

static int march_resident_ctas(int fmt) {
    static int cache[4][64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || fmt < 0 || fmt > 3) return kSMs;
    int &c = cache[fmt][dev];
    if (c == 0) {
        int sms = 0, nb = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (fmt == YAS_VOXEL_F32)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_persistent_kernel<YAS_VOXEL_F32>, 128, 0);
        else if (fmt == YAS_VOXEL_F16)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_persistent_kernel<YAS_VOXEL_F16>, 128, 0);
        else if (fmt == YAS_VOXEL_S16)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_persistent_kernel<YAS_VOXEL_S16>, 128, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_persistent_kernel<YAS_VOXEL_S24>, 128, 0);
        cudaGetLastError();
        c = std::max(1, nb) * std::max(1, sms);
    }
    return c;
}

static void launch_march_persistent(const MapDev &m, int fmt, const Cam &cam, const PosePair *P,
                                    const RaycastBuffers &rb, float4 *vmap, int vmap_pitch_elems, const int *skip,
                                    cudaStream_t s) {
    const unsigned total = (unsigned)(((cam.w + 7) / 8) * ((cam.h + 3) / 4) * 32);
    const int grid = std::min(march_resident_ctas(fmt), (int)((total + 127) / 128));
    switch (fmt) {
        case YAS_VOXEL_F32:
            march_persistent_kernel<YAS_VOXEL_F32><<<grid, 128, 0, s>>>(m, cam, P, rb.znear, rb.zfar, rb.zw, vmap,
                                                                        vmap_pitch_elems, skip, rb.queue, total, rb.fnear, rb.fw);
            break;
        case YAS_VOXEL_F16:
            march_persistent_kernel<YAS_VOXEL_F16><<<grid, 128, 0, s>>>(m, cam, P, rb.znear, rb.zfar, rb.zw, vmap,
                                                                        vmap_pitch_elems, skip, rb.queue, total, rb.fnear, rb.fw);
            break;
        case YAS_VOXEL_S16:
            march_persistent_kernel<YAS_VOXEL_S16><<<grid, 128, 0, s>>>(m, cam, P, rb.znear, rb.zfar, rb.zw, vmap,
                                                                        vmap_pitch_elems, skip, rb.queue, total, rb.fnear, rb.fw);
            break;
        default:
            march_persistent_kernel<YAS_VOXEL_S24><<<grid, 128, 0, s>>>(m, cam, P, rb.znear, rb.zfar, rb.zw, vmap,
                                                                        vmap_pitch_elems, skip, rb.queue, total, rb.fnear, rb.fw);
            break;
    }
}

template <int WX, int WY>
static void launch_march_tile(const MapDev &m, int fmt, const Cam &cam, const PosePair *P, const RaycastBuffers &rb,
                              float4 *vmap, int vmap_pitch_elems, const int *skip, cudaStream_t s) {
    dim3 grid((cam.w + 8 * WX - 1) / (8 * WX), (cam.h + 4 * WY - 1) / (4 * WY));
    const int threads = 32 * WX * WY;
    switch (fmt) {
        case YAS_VOXEL_F32:
            march_kernel<YAS_VOXEL_F32, WX, WY><<<grid, threads, 0, s>>>(m, cam, P, rb.znear, rb.zfar, rb.zw, vmap,
                                                                         vmap_pitch_elems, skip, rb.fnear, rb.fw);
            break;
        case YAS_VOXEL_F16:
            march_kernel<YAS_VOXEL_F16, WX, WY><<<grid, threads, 0, s>>>(m, cam, P, rb.znear, rb.zfar, rb.zw, vmap,
                                                                         vmap_pitch_elems, skip, rb.fnear, rb.fw);
            break;
        case YAS_VOXEL_S16:
            march_kernel<YAS_VOXEL_S16, WX, WY><<<grid, threads, 0, s>>>(m, cam, P, rb.znear, rb.zfar, rb.zw, vmap,
                                                                         vmap_pitch_elems, skip, rb.fnear, rb.fw);
            break;
        default:
            march_kernel<YAS_VOXEL_S24, WX, WY><<<grid, threads, 0, s>>>(m, cam, P, rb.znear, rb.zfar, rb.zw, vmap,
                                                                         vmap_pitch_elems, skip, rb.fnear, rb.fw);
            break;
    }
}

void launch_march(const MapDev &m, int fmt, const Cam &cam, const PosePair *P, const RaycastBuffers &rb,
                  float4 *vmap, int vmap_pitch_elems, const int *skip, cudaStream_t s, int tile) {
    switch (tile) {
        case 0: launch_march_persistent(m, fmt, cam, P, rb, vmap, vmap_pitch_elems, skip, s); break;
        case 1: launch_march_tile<1, 4>(m, fmt, cam, P, rb, vmap, vmap_pitch_elems, skip, s); break;
        case 4: launch_march_tile<4, 1>(m, fmt, cam, P, rb, vmap, vmap_pitch_elems, skip, s); break;
        default: launch_march_tile<2, 2>(m, fmt, cam, P, rb, vmap, vmap_pitch_elems, skip, s); break;
    }
}

__global__ void vmap_to_depth_kernel(const float4 *vmap, int vpitch, float *depth, int dpitch, int w,
                                     int h) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= w || y >= h) return;
    float4 v = vmap[(size_t)y * vpitch + x];
    depth[(size_t)y * dpitch + x] = v.w > 0.0f ? v.z : 0.0f;
}

void launch_vmap_to_depth(const float4 *vmap, int vpitch, float *depth, int dpitch, int w, int h,
                          cudaStream_t s) {
    dim3 grid((w + 127) / 128, h);
    vmap_to_depth_kernel<<<grid, 128, 0, s>>>(vmap, vpitch, depth, dpitch, w, h);
}

}  // namespace yas
