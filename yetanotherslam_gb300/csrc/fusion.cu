// fusion.cu — submap fusion, capacity growth and pose-correction
// re-integration.
//
// Reference semantics (paths relative to the reference project root):
//   MapStruct::Fuse(MapStruct*)   RGBDFusion/src/VoxelMap.cu:398-444: an empty
//                                 destination takes the source's storage
//                                 (Swap, :173-199); otherwise capacity for both
//                                 maps is reserved, then
//   CreateBlockFunctor            :231-262: every observed source voxel, moved
//                                 into the destination frame, allocates the
//                                 destination block that contains it;
//   MapStructFusionFunctor        :363-396: every destination voxel, moved into
//                                 the source frame, takes the trilinear source
//                                 sdf (all eight corners observed, the lerp
//                                 order of InterpolateSDF :305-361) with the
//                                 weight of the first corner:
//                                 sdf <- (sdf w + s ws) / (w + ws),
//                                 w <- min(255, w + ws);
//                                 then the source is released.
//   MapStruct::Reserve            :479-515: a larger table and pool, every block
//                                 re-inserted.
// Poses: GetPose() is the submap's pose in the world (Tcw of its keyframe), so
// source -> destination is inv(T_dst) * T_src.
//
// GB300 design: the pool is bump-allocated and a block's pool index never
// changes, so growing a map copies the pool prefix as it is and rebuilds the
// hash table from the block keys.  Block allocation reuses the warp-aggregated
// insert of the depth allocator; allocation decisions use the canonical FP32
// arithmetic of the rest of the map (one rounding per operation, fixed order).
#include "yas_internal.h"

namespace yas {

// Re-inserts blocks [0, n) into m's (empty) table with their pool indices.
__global__ void rehash_kernel(MapDev m, unsigned n) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned slot = 0;
        const int c = claim_slot(m, m.block_keys[i], &slot);
        if (c == 1) m.slots[slot].ptr = (int)i;
        else if (c < 0) raise_error(m, YAS_ERR_TABLE_FULL);
    }
}

// CreateBlockFunctor: one warp per 32-voxel slice of a source block.
template <int FMT>
__global__ void __launch_bounds__(256) fuse_alloc_kernel(MapDev dst, MapDev src, Rigid32 T, unsigned nsrc) {
    typedef VoxelIO<FMT> IO;
    const typename IO::T *vox = static_cast<const typename IO::T *>(src.voxels);
    const unsigned lane = lane_id();
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const float vs = dst.voxel_size;
    const float lim = 8.0f * (float)kCoordMax;
    for (unsigned w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nsrc * 16u; w += nwarps) {
        const unsigned b = w >> 4;
        const int li = (int)((w & 15u) * 32u + lane);  // z * 64 + y * 8 + x
        int bx, by, bz;
        unpack_key(src.block_keys[b], bx, by, bz);
        bool has = IO::wt(vox[(size_t)b * kBlockVoxels + li]) != 0;
        unsigned long long key = kEmptyKey;
        if (has) {
            const float px = cmul((float)(bx * 8 + (li & 7)), vs);
            const float py = cmul((float)(by * 8 + ((li >> 3) & 7)), vs);
            const float pz = cmul((float)(bz * 8 + (li >> 6)), vs);
            const float3 p = rigid_exact(T, px, py, pz);
            const float fx = floorf(cdiv(p.x, vs)), fy = floorf(cdiv(p.y, vs)), fz = floorf(cdiv(p.z, vs));
            if (fabsf(fx) < lim && fabsf(fy) < lim && fabsf(fz) < lim) {
                key = pack_key(floor_div8((int)fx), floor_div8((int)fy), floor_div8((int)fz));
            } else {
                raise_error(dst, YAS_ERR_COORD_RANGE);
                has = false;
            }
        }
        warp_insert<IO::kBytes>(dst, key, has);
    }
}

// Source voxel (x, y, z): sdf and weight, weight 0 if unobserved or absent.
template <int FMT>
struct SrcReader {
    typedef VoxelIO<FMT> IO;
    const MapDev &m;
    unsigned long long ckey = kEmptyKey;
    int cptr = -1;
    __device__ __forceinline__ explicit SrcReader(const MapDev &mm) : m(mm) {}
    __device__ __forceinline__ float read(int x, int y, int z, int &wt) {
        const int bx = x >> 3, by = y >> 3, bz = z >> 3;
        if (!coord_in_range(bx, by, bz)) {
            wt = 0;
            return 1.0f;
        }
        const unsigned long long k = pack_key(bx, by, bz);
        if (k != ckey) {
            ckey = k;
            cptr = find_block(m, k);
        }
        if (cptr < 0) {
            wt = 0;
            return 1.0f;
        }
        const typename IO::T v = __ldg(static_cast<const typename IO::T *>(m.voxels) + (size_t)cptr * kBlockVoxels +
                                       ((z & 7) << 6) + ((y & 7) << 3) + (x & 7));
        wt = IO::wt(v);
        return wt ? IO::sdf(v) : 1.0f;
    }
};

// MapStructFusionFunctor: one thread per destination voxel, over every
// destination block (the count is read after the allocation kernel).
template <int FMT>
__global__ void __launch_bounds__(256) fuse_blend_kernel(MapDev dst, MapDev src, Rigid32 T) {
    typedef VoxelIO<FMT> IO;
    const unsigned ndst = num_blocks(dst);
    typename IO::T *vox = static_cast<typename IO::T *>(dst.voxels);
    const float vs = dst.voxel_size;
    const float lim = 8.0f * (float)kCoordMax;
    SrcReader<FMT> rd(src);
    const size_t total = (size_t)ndst * kBlockVoxels;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const unsigned b = (unsigned)(i >> 9);
        const int li = (int)(i & 511);
        int bx, by, bz;
        unpack_key(dst.block_keys[b], bx, by, bz);
        const float3 p = rigid_exact(T, cmul((float)(bx * 8 + (li & 7)), vs), cmul((float)(by * 8 + ((li >> 3) & 7)), vs),
                                     cmul((float)(bz * 8 + (li >> 6)), vs));
        const float qx = cdiv(p.x, vs), qy = cdiv(p.y, vs), qz = cdiv(p.z, vs);
        const float fx = floorf(qx), fy = floorf(qy), fz = floorf(qz);
        if (!(fabsf(fx) < lim && fabsf(fy) < lim && fabsf(fz) < lim)) continue;
        const int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
        const float ax = qx - fx, ay = qy - fy, az = qz - fz;
        // corners in InterpolateSDF's order; the first unobserved one ends it
        int w0, w;
        const float s000 = rd.read(x0, y0, z0, w0);
        if (!w0) continue;
        const float s100 = rd.read(x0 + 1, y0, z0, w);
        if (!w) continue;
        const float s010 = rd.read(x0, y0 + 1, z0, w);
        if (!w) continue;
        const float s110 = rd.read(x0 + 1, y0 + 1, z0, w);
        if (!w) continue;
        const float s001 = rd.read(x0, y0, z0 + 1, w);
        if (!w) continue;
        const float s101 = rd.read(x0 + 1, y0, z0 + 1, w);
        if (!w) continue;
        const float s011 = rd.read(x0, y0 + 1, z0 + 1, w);
        if (!w) continue;
        const float s111 = rd.read(x0 + 1, y0 + 1, z0 + 1, w);
        if (!w) continue;
        const float r0 = s000 * (1.0f - ax) + s100 * ax;
        const float r1 = r0 * (1.0f - ay) + (s010 * (1.0f - ax) + s110 * ax) * ay;
        const float r2 = s001 * (1.0f - ax) + s101 * ax;
        const float s = r1 * (1.0f - az) + (r2 * (1.0f - ay) + (s011 * (1.0f - ax) + s111 * ax) * ay) * az;
        typename IO::T &d = vox[i];
        const int dw = IO::wt(d);
        const float ds = dw ? IO::sdf(d) : 0.0f;
        const float ns = (ds * (float)dw + s * (float)w0) / (float)(dw + w0);
        d = IO::make(ns, min(dst.max_weight, dw + w0));
    }
}

void launch_rehash(const MapDev &m, unsigned n, cudaStream_t s) {
    if (n) rehash_kernel<<<(n + 255) / 256, 256, 0, s>>>(m, n);
}

void launch_fuse_alloc(const MapDev &dst, const MapDev &src, int fmt, const Rigid32 &T_src_dst, unsigned nsrc,
                       cudaStream_t s) {
    const int grid = kSMs * 8;
    switch (fmt) {
        case YAS_VOXEL_F32:
            fuse_alloc_kernel<YAS_VOXEL_F32><<<grid, 256, 0, s>>>(dst, src, T_src_dst, nsrc);
            break;
        case YAS_VOXEL_F16:
            fuse_alloc_kernel<YAS_VOXEL_F16><<<grid, 256, 0, s>>>(dst, src, T_src_dst, nsrc);
            break;
        case YAS_VOXEL_S16:
            fuse_alloc_kernel<YAS_VOXEL_S16><<<grid, 256, 0, s>>>(dst, src, T_src_dst, nsrc);
            break;
        default:
            fuse_alloc_kernel<YAS_VOXEL_S24><<<grid, 256, 0, s>>>(dst, src, T_src_dst, nsrc);
            break;
    }
}

void launch_fuse_blend(const MapDev &dst, const MapDev &src, int fmt, const Rigid32 &T_dst_src, cudaStream_t s) {
    const int grid = kSMs * 8;
    switch (fmt) {
        case YAS_VOXEL_F32:
            fuse_blend_kernel<YAS_VOXEL_F32><<<grid, 256, 0, s>>>(dst, src, T_dst_src);
            break;
        case YAS_VOXEL_F16:
            fuse_blend_kernel<YAS_VOXEL_F16><<<grid, 256, 0, s>>>(dst, src, T_dst_src);
            break;
        case YAS_VOXEL_S16:
            fuse_blend_kernel<YAS_VOXEL_S16><<<grid, 256, 0, s>>>(dst, src, T_dst_src);
            break;
        default:
            fuse_blend_kernel<YAS_VOXEL_S24><<<grid, 256, 0, s>>>(dst, src, T_dst_src);
            break;
    }
}

}  // namespace yas
