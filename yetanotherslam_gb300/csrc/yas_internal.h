// yas_internal.h — host-side structures shared by the translation units of
// libyas_gb300: handle layouts, pose algebra, camera parameters and the
// launch wrappers each .cu file provides.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "yas_common.cuh"

#define YAS_TRY_CUDA(expr)                                             \
    do {                                                               \
        cudaError_t e_ = (expr);                                       \
        if (e_ != cudaSuccess) {                                       \
            ::yas::record_cuda_error(e_, #expr, __FILE__, __LINE__);   \
            return YAS_ERR_CUDA;                                       \
        }                                                              \
    } while (0)

#define YAS_TRY(expr)               \
    do {                            \
        int s_ = (expr);            \
        if (s_ != YAS_OK) return s_; \
    } while (0)

namespace yas {

void record_cuda_error(cudaError_t e, const char *expr, const char *file, int line);

// ------------------------------------------------------------------ poses
struct Pose64 {
    double r[9];
    double t[3];
};

Pose64 pose_identity();
Pose64 pose_from(const yas_pose &p);
yas_pose pose_to(const Pose64 &p);
// inverse: R^T, -(R^T t) with t_i' = -((R0i t0 + R1i t1) + R2i t2)
Pose64 pose_inverse(const Pose64 &p);
Pose64 pose_mul(const Pose64 &a, const Pose64 &b);
Rigid32 rigid_from(const Pose64 &p);  // element-wise round to nearest float

// A pose pair as kernels read it from device memory.
struct __align__(16) PosePair {
    Rigid32 T;     // camera -> map
    Rigid32 Tinv;  // map -> camera
};

// ------------------------------------------------------------------ camera
struct Cam {
    float fx, fy, cx, cy;
    float invfx, invfy;  // (float)(1.0 / fx)
    int w, h;
};
Cam make_cam(float fx, float fy, float cx, float cy, int w, int h);

// ------------------------------------------------------------------ map.cu
int map_dev_alloc(yas_map *m);
void map_dev_free(yas_map *m);
MapDev map_view(const yas_map *m);

// `dependent` (allocate, visible, integrate): launched as a programmatic
// dependent of the previous kernel on `s`, which must be a kernel; its CTAs
// are scheduled while that kernel finishes and wait for it in the kernel.
// Allocates blocks along each depth ray (FP32-exact line tracing).
void launch_allocate(const MapDev &m, int fmt, const float *depth, int pitch_elems, const Cam &cam,
                     const PosePair *P, const int *skip, cudaStream_t s, bool dependent = false);
// Compacts the visible blocks into m.visible; hdr->n_visible must be zero.
void launch_visible(const MapDev &m, const Cam &cam, const PosePair *P, const int *skip,
                    cudaStream_t s, bool dependent = false);
// Integrates depth into the visible blocks.
// `grid_ctas` 0: the default grid (152 x 8 CTAs of 256 threads).
void launch_integrate(const MapDev &m, int fmt, const float *depth, int pitch_elems, const Cam &cam,
                      const PosePair *P, const int *skip, cudaStream_t s, int grid_ctas = 0,
                      bool dependent = false);
void launch_deintegrate(const MapDev &m, int fmt, const float *depth, int pitch_elems, const Cam &cam,
                        const PosePair *P, cudaStream_t s);
// Submap fusion and growth (fusion.cu)
void launch_rehash(const MapDev &m, unsigned n, cudaStream_t s);
void launch_fuse_alloc(const MapDev &dst, const MapDev &src, int fmt, const Rigid32 &T_src_dst, unsigned nsrc,
                       cudaStream_t s);
void launch_fuse_blend(const MapDev &dst, const MapDev &src, int fmt, const Rigid32 &T_dst_src, cudaStream_t s);
void launch_map_reset(const MapDev &m, cudaStream_t s);
void launch_map_export(const MapDev &m, int fmt, int *coords, float *sdf, float *wt, unsigned first,
                       unsigned count, cudaStream_t s);
void launch_map_import(const MapDev &m, int fmt, const int *coords, const float *sdf, const float *wt,
                       unsigned count, cudaStream_t s);
void launch_visible_coords(const MapDev &m, int *coords, unsigned count, cudaStream_t s);

// ------------------------------------------------------------------ raycast.cu
struct RaycastBuffers {
    int w, h;          // image size
    int zw, zh;        // z-range map size: ceil(w/8), ceil(h/8)
    float *znear;      // zw*zh
    float *zfar;       // zw*zh
    unsigned *queue;   // next pixel of the persistent march (reset with the z-range)
    int fw, fh;        // fine near-bound map size: ceil(w/4), ceil(h/4)
    float *fnear;      // fw*fh: nearest visible block whose projected box covers the 4x4 pixels
};
void launch_zrange(const MapDev &m, const Cam &cam, const PosePair *P, RaycastBuffers &rb,
                   const int *skip, cudaStream_t s);
// `warps_x` 1, 2 (the default), 4: one thread per pixel, a 128-thread CTA's
// four 8x4-pixel warp tiles side by side in x (8x16, 16x8, 32x4 pixels);
// 0: persistent warps taking 8x4-pixel tiles from a queue.  The output is
// the same.
void launch_march(const MapDev &m, int fmt, const Cam &cam, const PosePair *P, const RaycastBuffers &rb,
                  float4 *vmap, int vmap_pitch_elems, const int *skip, cudaStream_t s, int warps_x = 2);
void launch_vmap_to_depth(const float4 *vmap, int vpitch, float *depth, int dpitch, int w, int h,
                          cudaStream_t s);

// ------------------------------------------------------------------ mesh.cu
void mesh_tables_upload();  // generates the marching-cubes tables once per device
struct MeshBuffers {
    int max_tris;
    float *points;     // 9 * max_tris
    float *normals;    // 9 * max_tris
    int *cases;        // max_tris
    int *cube_xyz;     // 3 * max_tris
    unsigned *block_tris;    // per block triangle count (max_blocks)
    unsigned *block_offset;  // exclusive scan (max_blocks + 1)
    unsigned *counters;      // [0] = total triangles
    size_t cap_blocks;
};
int mesher_ensure_blocks(MeshBuffers &mb, size_t n_blocks);
int launch_meshify(const MapDev &m, int fmt, MeshBuffers &mb, unsigned n_blocks, cudaStream_t s);

}  // namespace yas

// ------------------------------------------------------------------ handles
struct yas_map {
    yas_map_config cfg;
    yas::Cam cam_K;  // intrinsics from MapStruct(K); w/h unused
    cudaStream_t stream = nullptr;
    // device
    yas::HashSlot *slots = nullptr;
    unsigned slot_mask = 0;
    unsigned long long *block_keys = nullptr;
    void *voxels = nullptr;
    int *visible = nullptr;
    yas::MapHeader *hdr = nullptr;
    yas::PosePair *pose_dev = nullptr;  // pose of the last fuse / visibility call
    yas::MapHeader *hdr_host = nullptr; // pinned mirror
    // host state (MapStruct::mTcw, mbActive, mbInHibernation)
    yas::Pose64 Tcw;
    std::mutex pose_mutex;
    bool active = true;
    std::mutex active_mutex;
    bool hibernated = false;
    std::vector<unsigned char> hib_slots, hib_keys, hib_voxels, hib_visible;
    yas::MapHeader hib_hdr;
    size_t voxel_bytes() const {
        return (size_t)cfg.max_blocks * yas::kBlockVoxels * (cfg.voxel_format == YAS_VOXEL_F32 ? 8 : 4);
    }
};

struct yas_raycaster {
    int w = 0, h = 0;
    yas::Cam cam;
    cudaStream_t stream = nullptr;
    yas::RaycastBuffers rb{};
    float4 *vmap = nullptr;  // w*h
    float *depth_tmp = nullptr;
    yas::PosePair *pose_dev = nullptr;
    unsigned last_visible = 0;
};

struct yas_mesher {
    cudaStream_t stream = nullptr;
    yas::MeshBuffers mb{};
    unsigned last_tris = 0;
};
