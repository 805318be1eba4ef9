// map.cu — voxel-hash TSDF map: block allocation, visibility compaction,
// depth integration, reset and host export/import.
//
// Reference semantics (paths relative to the reference project root):
//   allocation   RGBDFusion/src/VoxelMap.cu:517-652 (CreateBlockLineTracingFunctor)
//   visibility   RGBDFusion/src/VoxelMap.cu:654-717, RGBDFusion/utils/VoxelStructUtils.h:112-147
//   integration  RGBDFusion/src/VoxelMap.cu:719-786 (DepthFusionFunctor)
//   reset        RGBDFusion/src/VoxelMap.cu:24-58
//
// GB300 layout: 16-byte open-addressing slots with packed 64-bit keys; the
// voxel pool is bump-allocated so pool index i <-> block_keys[i] is itself
// the allocated-block list (no full-table scans); new blocks are zeroed by the
// warp that allocated them.
#include "yas_internal.h"

namespace yas {

// f2i_floor: floor to int with NaN/out-of-range mapped to INT_MIN; the CPU
// oracle uses the same rule so that degenerate projections agree.
__device__ __forceinline__ int f2i_floor(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return (int)0x80000000;
    return (int)floorf(x);
}

// ---------------------------------------------------------------- allocation
// Block coordinate of a camera-ray point at metric depth z (FP32 canonical):
// UnProjectWorld (VoxelStructUtils.h:100-110) -> WorldPtToVoxelPos -> VoxelPosToBlockPos.
__device__ __forceinline__ void ray_block(const Cam &c, const Rigid32 &T, float vs, int x, int y,
                                          float z, int b[3]) {
    float px = cmul(cmul(c.invfx, csub((float)x, c.cx)), z);
    float py = cmul(cmul(c.invfy, csub((float)y, c.cy)), z);
    float3 q = rigid_exact(T, px, py, z);
    b[0] = floor_div8(f2i_floor(cdiv(q.x, vs)));
    b[1] = floor_div8(f2i_floor(cdiv(q.y, vs)));
    b[2] = floor_div8(f2i_floor(cdiv(q.z, vs)));
}

// 3-D Bresenham walker over block coordinates with the reference's major-axis
// choice and error terms (VoxelMap.cu:568-650).
struct BlockLine {
    int cur[3];
    int inc[3];
    int d2[3];   // 2*|d|
    int major, a1, a2;
    int err1, err2;
    int count;   // number of blocks on the line (|d_major| + 1)

    __device__ __forceinline__ void init(const int s[3], const int e[3]) {
        int ad[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            int d = e[i] - s[i];
            cur[i] = s[i];
            inc[i] = d < 0 ? -1 : 1;
            ad[i] = d < 0 ? -d : d;
            d2[i] = ad[i] << 1;
        }
        if (ad[0] >= ad[1] && ad[0] >= ad[2]) {
            major = 0; a1 = 1; a2 = 2;
        } else if (ad[1] >= ad[0] && ad[1] >= ad[2]) {
            major = 1; a1 = 0; a2 = 2;
        } else {
            major = 2; a1 = 1; a2 = 0;
        }
        err1 = d2[a1] - 1;
        err2 = d2[a2] - 1;
        count = ad[major] + 1;
    }
    __device__ __forceinline__ void step() {
        if (err1 > 0) {
            cur[a1] += inc[a1];
            err1 -= d2[major];
        }
        if (err2 > 0) {
            cur[a2] += inc[a2];
            err2 -= d2[major];
        }
        err1 += d2[a1];
        err2 += d2[a2];
        cur[major] += inc[major];
    }
};

constexpr int kMaxLineBlocks = 1024;

// Launches `k` on `s`; `dependent`: as a programmatic dependent of the
// previous kernel on `s` (the kernel calls dependent_wait() first).
template <typename... P, typename... A>
static void launch_kernel(void (*k)(P...), dim3 grid, dim3 block, cudaStream_t s, bool dependent, A... args) {
    cudaLaunchConfig_t c = {};
    c.gridDim = grid;
    c.blockDim = block;
    c.dynamicSmemBytes = 0;
    c.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = at;
    c.numAttrs = dependent ? 1 : 0;
    cudaLaunchKernelEx(&c, k, args...);
}

template <int VBYTES>
__global__ void __launch_bounds__(256) allocate_kernel(MapDev m, const float *__restrict__ depth,
                                                       int pitch, Cam cam, const PosePair *P,
                                                       const int *skip) {
    dependent_wait();
    release_dependents();
    if (skip && *skip) return;
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    const Rigid32 T = P->T;

    BlockLine line;
    int n = 0;
    if (x < cam.w && y < cam.h) {
        float dist = depth[(size_t)y * pitch + x];
        if (!(isnan(dist) || dist < m.depth_min || dist > m.depth_max)) {
            const float half = m.trunc * 0.5f;
            float dnear = fmaxf(m.depth_min, csub(dist, half));
            float dfar = fminf(m.depth_max, cadd(dist, half));
            if (dnear < dfar) {
                int bs[3], be[3];
                ray_block(cam, T, m.voxel_size, x, y, dnear, bs);
                ray_block(cam, T, m.voxel_size, x, y, dfar, be);
                line.init(bs, be);
                n = line.count;
                if (n > kMaxLineBlocks) {
                    raise_error(m, YAS_ERR_COORD_RANGE);
                    n = 0;
                }
            }
        }
    }
    const int nmax = __reduce_max_sync(0xffffffffu, n);
    for (int s = 0; s < nmax; ++s) {
        bool has = s < n;
        unsigned long long key = kEmptyKey;
        if (has) {
            if (s > 0) line.step();
            if (coord_in_range(line.cur[0], line.cur[1], line.cur[2])) {
                key = pack_key(line.cur[0], line.cur[1], line.cur[2]);
            } else {
                raise_error(m, YAS_ERR_COORD_RANGE);
                has = false;
            }
        }
        warp_insert<VBYTES>(m, key, has);
    }
}

void launch_allocate(const MapDev &m, int fmt, const float *depth, int pitch_elems, const Cam &cam,
                     const PosePair *P, const int *skip, cudaStream_t s, bool dependent) {
    dim3 block(256);
    dim3 grid((cam.w + 31) / 32, (cam.h + 7) / 8);
    launch_kernel(fmt == YAS_VOXEL_F32 ? allocate_kernel<8> : allocate_kernel<4>, grid, block, s, dependent, m,
                  depth, pitch_elems, cam, P, skip);
}

// ---------------------------------------------------------------- visibility
// CheckBlockVisibility (VoxelStructUtils.h:112-147), FP32 canonical.
__device__ __forceinline__ bool block_visible(const Cam &c, const Rigid32 &Tinv, float vs, float dmin,
                                              float dmax, int bx, int by, int bz) {
    const float scale = cmul(vs, 8.0f);
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
        float wx = cmul((float)(bx + (corner & 1)), scale);
        float wy = cmul((float)(by + ((corner >> 1) & 1)), scale);
        float wz = cmul((float)(bz + ((corner >> 2) & 1)), scale);
        float3 p = rigid_exact(Tinv, wx, wy, wz);
        float u = cadd(cdiv(cmul(c.fx, p.x), p.z), c.cx);
        float v = cadd(cdiv(cmul(c.fy, p.y), p.z), c.cy);
        if (!(u < 0.0f || v < 0.0f || u > (float)(c.w - 1) || v > (float)(c.h - 1) || p.z < dmin ||
              p.z > dmax))
            return true;
    }
    return false;
}

__global__ void __launch_bounds__(256) visible_kernel(MapDev m, Cam cam, const PosePair *P,
                                                      const int *skip) {
    dependent_wait();
    release_dependents();
    if (skip && *skip) return;
    const unsigned n = num_blocks(m);
    const Rigid32 Tinv = P->Tinv;
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        unsigned i = base + lane_id();
        bool vis = false;
        if (i < n) {
            int bx, by, bz;
            unpack_key(m.block_keys[i], bx, by, bz);
            vis = block_visible(cam, Tinv, m.voxel_size, m.depth_min, m.depth_max, bx, by, bz);
        }
        unsigned slot = warp_append(&m.hdr->n_visible, vis);
        if (vis) m.visible[slot] = (int)i;
    }
}

void launch_visible(const MapDev &m, const Cam &cam, const PosePair *P, const int *skip,
                    cudaStream_t s, bool dependent) {
    launch_kernel(visible_kernel, dim3(kSMs * 4), dim3(256), s, dependent, m, cam, P, skip);
}

// ---------------------------------------------------------------- integration
// Pixel index floor(((a / z) + c) + 0.5) with the IEEE quotient a / z, as the
// canonical FP32 order defines it.  The quotient is first formed as a * (1/z)
// with the correctly rounded reciprocal (within 2 ulp of a / z); only when the
// resulting coordinate lies within 8 ulp of an integer, where the two could
// round to different pixels, is the exact division evaluated.
__device__ __forceinline__ int project_exact(float a, float z, float rz, float c) {
    const float t = cadd(cadd(cmul(a, rz), c), 0.5f);
    const float ft = floorf(t);
    const float tol = 8.0f * fmaxf(fabsf(t), fabsf(t - c)) * 1.1920929e-7f;
    if (fabsf(t) < 8.0e6f && t - ft > tol && ft + 1.0f - t > tol) return (int)ft;
    return f2i_floor(cadd(cadd(cdiv(a, z), c), 0.5f));
}

// Each 128-thread group owns one block; thread t updates voxels 4t..4t+3
// (z = t/16, y = (t/2)%8, x = 4*(t%2) .. +3), one 16-byte (or 32-byte) access.
// SIGN = +1: DepthFusionFunctor (VoxelMap.cu:719-786).  SIGN = -1: the same
// observation removed again (de-integration, for re-integration after a pose
// correction): s <- (s w - d) / (w - 1), w <- w - 1; exact while the weight
// stayed below the cap, as the reference's running average is then invertible.
template <int FMT, int SIGN>
__global__ void __launch_bounds__(256) integrate_kernel(MapDev m, const float *__restrict__ depth,
                                                        int pitch, Cam cam, const PosePair *P,
                                                        const int *skip) {
    typedef VoxelIO<FMT> IO;
    typedef typename IO::T V;
    dependent_wait();
    if (skip && *skip) return;
    const unsigned nvis = *(volatile unsigned *)&m.hdr->n_visible;
    const Rigid32 Tinv = P->Tinv;
    const int t = threadIdx.x & 127;
    const int lz = t >> 4, ly = (t >> 1) & 7, lx0 = (t & 1) * 4;
    const float vs = m.voxel_size, inv_trunc = 1.0f / m.trunc, ntrunc = -m.trunc;
    V *vox = static_cast<V *>(m.voxels);
    for (unsigned j = blockIdx.x * 2 + (threadIdx.x >> 7); j < nvis; j += gridDim.x * 2) {
        const int b = m.visible[j];
        int bx, by, bz;
        unpack_key(m.block_keys[b], bx, by, bz);
        V *p = vox + (size_t)b * kBlockVoxels + t * 4;
        V v[4];
        if (sizeof(V) == 4) {
            uint4 q = *reinterpret_cast<const uint4 *>(p);
            v[0] = *reinterpret_cast<V *>(&q.x);
            v[1] = *reinterpret_cast<V *>(&q.y);
            v[2] = *reinterpret_cast<V *>(&q.z);
            v[3] = *reinterpret_cast<V *>(&q.w);
        } else {
            float4 q0 = reinterpret_cast<const float4 *>(p)[0];
            float4 q1 = reinterpret_cast<const float4 *>(p)[1];
            v[0] = *reinterpret_cast<V *>(&q0.x);
            v[1] = *reinterpret_cast<V *>(&q0.z);
            v[2] = *reinterpret_cast<V *>(&q1.x);
            v[3] = *reinterpret_cast<V *>(&q1.z);
        }
        const float wy = cmul((float)(by * 8 + ly), vs);
        const float wz = cmul((float)(bz * 8 + lz), vs);
        bool dirty = false;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float wx = cmul((float)(bx * 8 + lx0 + q), vs);
            float3 pc = rigid_exact(Tinv, wx, wy, wz);
            const float rz = __frcp_rn(pc.z);
            int u = project_exact(cmul(cam.fx, pc.x), pc.z, rz, cam.cx);
            int vv = project_exact(cmul(cam.fy, pc.y), pc.z, rz, cam.cy);
            if (u < 0 || vv < 0 || u > cam.w - 1 || vv > cam.h - 1) continue;
            float dist = __ldg(depth + (size_t)vv * pitch + u);
            if (isnan(dist) || dist > m.depth_max || dist < m.depth_min) continue;
            float sdf = csub(dist, pc.z);
            if (sdf < ntrunc) continue;
            sdf = fminf(1.0f, sdf * inv_trunc);
            int w = IO::wt(v[q]);
            float ns;
            if (SIGN > 0) {
                if (w == 0) {
                    ns = sdf;
                    w = 1;
                } else {
                    ns = __fdividef(fmaf(IO::sdf(v[q]), (float)w, sdf), (float)(w + 1));
                    w = min(m.max_weight, w + 1);
                }
            } else {
                if (w == 0) continue;
                if (w == 1) {
                    ns = 0.0f;
                    w = 0;
                } else {
                    ns = __fdividef(fmaf(IO::sdf(v[q]), (float)w, -sdf), (float)(w - 1));
                    w = w - 1;
                }
            }
            v[q] = IO::make(ns, w);
            dirty = true;
        }
        if (dirty) {
            if (sizeof(V) == 4) {
                uint4 q;
                q.x = *reinterpret_cast<unsigned *>(&v[0]);
                q.y = *reinterpret_cast<unsigned *>(&v[1]);
                q.z = *reinterpret_cast<unsigned *>(&v[2]);
                q.w = *reinterpret_cast<unsigned *>(&v[3]);
                *reinterpret_cast<uint4 *>(p) = q;
            } else {
                float4 q0, q1;
                *reinterpret_cast<V *>(&q0.x) = v[0];
                *reinterpret_cast<V *>(&q0.z) = v[1];
                *reinterpret_cast<V *>(&q1.x) = v[2];
                *reinterpret_cast<V *>(&q1.z) = v[3];
                reinterpret_cast<float4 *>(p)[0] = q0;
                reinterpret_cast<float4 *>(p)[1] = q1;
            }
        }
    }
}

template <int SIGN>
static void launch_integrate_sign(const MapDev &m, int fmt, const float *depth, int pitch_elems, const Cam &cam,
                                  const PosePair *P, const int *skip, cudaStream_t s, int grid_ctas = 0,
                                  bool dependent = false) {
    const dim3 grid(grid_ctas > 0 ? grid_ctas : kSMs * 8);
    switch (fmt) {
        case YAS_VOXEL_F32:
            launch_kernel(integrate_kernel<YAS_VOXEL_F32, SIGN>, grid, dim3(256), s, dependent, m, depth, pitch_elems,
                          cam, P, skip);
            break;
        case YAS_VOXEL_F16:
            launch_kernel(integrate_kernel<YAS_VOXEL_F16, SIGN>, grid, dim3(256), s, dependent, m, depth, pitch_elems,
                          cam, P, skip);
            break;
        case YAS_VOXEL_S16:
            launch_kernel(integrate_kernel<YAS_VOXEL_S16, SIGN>, grid, dim3(256), s, dependent, m, depth, pitch_elems,
                          cam, P, skip);
            break;
        default:
            launch_kernel(integrate_kernel<YAS_VOXEL_S24, SIGN>, grid, dim3(256), s, dependent, m, depth, pitch_elems,
                          cam, P, skip);
            break;
    }
}

void launch_integrate(const MapDev &m, int fmt, const float *depth, int pitch_elems, const Cam &cam,
                      const PosePair *P, const int *skip, cudaStream_t s, int grid_ctas, bool dependent) {
    launch_integrate_sign<1>(m, fmt, depth, pitch_elems, cam, P, skip, s, grid_ctas, dependent);
}

void launch_deintegrate(const MapDev &m, int fmt, const float *depth, int pitch_elems, const Cam &cam,
                        const PosePair *P, cudaStream_t s) {
    launch_integrate_sign<-1>(m, fmt, depth, pitch_elems, cam, P, nullptr, s);
}

// ---------------------------------------------------------------- reset
__global__ void reset_slots_kernel(MapDev m) {
    const unsigned n = m.slot_mask + 1;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        HashSlot s;
        s.key = kEmptyKey;
        s.ptr = -1;
        s.pad = 0;
        m.slots[i] = s;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        MapHeader h = {};
        *m.hdr = h;
    }
}

void launch_map_reset(const MapDev &m, cudaStream_t s) {
    reset_slots_kernel<<<kSMs * 4, 256, 0, s>>>(m);
}

// ---------------------------------------------------------------- export/import
template <int FMT>
__global__ void export_kernel(MapDev m, int *coords, float *sdf, float *wt, unsigned first,
                              unsigned count) {
    typedef VoxelIO<FMT> IO;
    const typename IO::T *vox = static_cast<const typename IO::T *>(m.voxels);
    for (unsigned j = blockIdx.x; j < count; j += gridDim.x) {
        unsigned b = first + j;
        if (threadIdx.x == 0) {
            int x, y, z;
            unpack_key(m.block_keys[b], x, y, z);
            coords[3 * j + 0] = x;
            coords[3 * j + 1] = y;
            coords[3 * j + 2] = z;
        }
        for (int i = threadIdx.x; i < kBlockVoxels; i += blockDim.x) {
            typename IO::T v = vox[(size_t)b * kBlockVoxels + i];
            sdf[(size_t)j * kBlockVoxels + i] = IO::sdf(v);
            wt[(size_t)j * kBlockVoxels + i] = (float)IO::wt(v);
        }
    }
}

void launch_map_export(const MapDev &m, int fmt, int *coords, float *sdf, float *wt, unsigned first,
                       unsigned count, cudaStream_t s) {
    if (count == 0) return;
    unsigned grid = count < 4096 ? count : 4096;
    if (fmt == YAS_VOXEL_F32)
        export_kernel<YAS_VOXEL_F32><<<grid, 128, 0, s>>>(m, coords, sdf, wt, first, count);
    else if (fmt == YAS_VOXEL_F16)
        export_kernel<YAS_VOXEL_F16><<<grid, 128, 0, s>>>(m, coords, sdf, wt, first, count);
    else if (fmt == YAS_VOXEL_S16)
        export_kernel<YAS_VOXEL_S16><<<grid, 128, 0, s>>>(m, coords, sdf, wt, first, count);
    else
        export_kernel<YAS_VOXEL_S24><<<grid, 128, 0, s>>>(m, coords, sdf, wt, first, count);
}

// One warp per imported block: lane 0 claims the slot and a pool index.
template <int FMT>
__global__ void import_kernel(MapDev m, const int *coords, const float *sdf, const float *wt,
                              unsigned count) {
    typedef VoxelIO<FMT> IO;
    typename IO::T *vox = static_cast<typename IO::T *>(m.voxels);
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned j = warp; j < count; j += nwarps) {
        int x = coords[3 * j], y = coords[3 * j + 1], z = coords[3 * j + 2];
        int b = -1;
        if (lane_id() == 0) {
            if (!coord_in_range(x, y, z)) {
                raise_error(m, YAS_ERR_COORD_RANGE);
            } else {
                unsigned long long key = pack_key(x, y, z);
                unsigned slot;
                int c = claim_slot(m, key, &slot);
                if (c == 1) {
                    unsigned idx = atomicAdd(&m.hdr->n_alloc, 1u);
                    if (idx < (unsigned)m.max_blocks) {
                        m.block_keys[idx] = key;
                        m.slots[slot].ptr = (int)idx;
                        b = (int)idx;
                    } else {
                        raise_error(m, YAS_ERR_POOL_FULL);
                    }
                } else if (c == 0) {
                    // Existing block: overwrite its contents. Its ptr was set by an
                    // earlier kernel, so the plain read is complete.
                    b = find_block(m, key);
                } else {
                    raise_error(m, YAS_ERR_TABLE_FULL);
                }
            }
        }
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b < 0) continue;
        for (int i = lane_id(); i < kBlockVoxels; i += 32) {
            float s = sdf[(size_t)j * kBlockVoxels + i];
            int w = (int)wt[(size_t)j * kBlockVoxels + i];
            vox[(size_t)b * kBlockVoxels + i] = IO::make(s, w);
        }
    }
}

void launch_map_import(const MapDev &m, int fmt, const int *coords, const float *sdf, const float *wt,
                       unsigned count, cudaStream_t s) {
    if (count == 0) return;
    if (fmt == YAS_VOXEL_F32)
        import_kernel<YAS_VOXEL_F32><<<256, 256, 0, s>>>(m, coords, sdf, wt, count);
    else if (fmt == YAS_VOXEL_F16)
        import_kernel<YAS_VOXEL_F16><<<256, 256, 0, s>>>(m, coords, sdf, wt, count);
    else if (fmt == YAS_VOXEL_S16)
        import_kernel<YAS_VOXEL_S16><<<256, 256, 0, s>>>(m, coords, sdf, wt, count);
    else
        import_kernel<YAS_VOXEL_S24><<<256, 256, 0, s>>>(m, coords, sdf, wt, count);
}

__global__ void visible_coords_kernel(MapDev m, int *coords, unsigned count) {
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
        int x, y, z;
        unpack_key(m.block_keys[m.visible[j]], x, y, z);
        coords[3 * j] = x;
        coords[3 * j + 1] = y;
        coords[3 * j + 2] = z;
    }
}

void launch_visible_coords(const MapDev &m, int *coords, unsigned count, cudaStream_t s) {
    if (count == 0) return;
    visible_coords_kernel<<<(count + 255) / 256, 256, 0, s>>>(m, coords, count);
}

// ---------------------------------------------------------------- device memory
MapDev map_view(const yas_map *m) {
    MapDev d;
    d.slots = m->slots;
    d.slot_mask = m->slot_mask;
    d.block_keys = m->block_keys;
    d.voxels = m->voxels;
    d.visible = m->visible;
    d.hdr = m->hdr;
    d.max_blocks = m->cfg.max_blocks;
    d.voxel_size = m->cfg.voxel_size;
    d.trunc = m->cfg.trunc_dist;
    d.depth_min = m->cfg.depth_min;
    d.depth_max = m->cfg.depth_max;
    d.max_weight = m->cfg.max_weight;
    return d;
}

int map_dev_alloc(yas_map *m) {
    const size_t nslots = (size_t)m->cfg.hash_slots;
    if (cudaMalloc(&m->slots, nslots * sizeof(HashSlot)) != cudaSuccess ||
        cudaMalloc(&m->block_keys, (size_t)m->cfg.max_blocks * sizeof(unsigned long long)) !=
            cudaSuccess ||
        cudaMalloc(&m->voxels, m->voxel_bytes()) != cudaSuccess ||
        cudaMalloc(&m->visible, (size_t)m->cfg.max_blocks * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&m->hdr, sizeof(MapHeader)) != cudaSuccess) {
        cudaGetLastError();
        map_dev_free(m);
        return YAS_ERR_OOM;
    }
    m->slot_mask = (unsigned)(nslots - 1);
    return YAS_OK;
}

void map_dev_free(yas_map *m) {
    cudaFree(m->slots);
    cudaFree(m->block_keys);
    cudaFree(m->voxels);
    cudaFree(m->visible);
    cudaFree(m->hdr);
    m->slots = nullptr;
    m->block_keys = nullptr;
    m->voxels = nullptr;
    m->visible = nullptr;
    m->hdr = nullptr;
}

}  // namespace yas
