/*
 * yas.h — C ABI of the GB300-native dense RGB-D path (voxel-hash TSDF fusion,
 * raycasting, marching cubes, dense ICP + photometric tracking).
 *
 * Every entry point is a plain C function over opaque handles, POD structs,
 * raw pointers and sizes.  Every call returns an int status (YAS_OK == 0).
 * Each handle owns one CUDA stream (`stream` at creation; NULL = the legacy
 * default stream) and every device operation of that handle is ordered on it.
 *
 * The handles mirror the classes of YetAnotherSLAM's RGBDFusion library; each
 * declaration cites the reference member it replaces (paths relative to the
 * reference project root).
 *
 * Pose convention: yas_pose is a row-major 3x4 [R|t] in double precision.
 * `Tcm` maps camera coordinates to map (submap) coordinates, as the
 * reference's Sophus::SE3d Tcm argument of MapStruct::Fuse / RayTrace.
 */
#ifndef YAS_H
#define YAS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define YAS_API __attribute__((visibility("default")))
#else
#define YAS_API
#endif

/* ---------------------------------------------------------------- status */
enum yas_status {
    YAS_OK = 0,
    YAS_ERR_BAD_ARG = 1,       /* null handle / bad size / bad enum          */
    YAS_ERR_OOM = 2,           /* device or pinned-host allocation failed    */
    YAS_ERR_CUDA = 3,          /* a CUDA runtime call failed                 */
    YAS_ERR_TABLE_FULL = 4,    /* hash probe limit reached on insert         */
    YAS_ERR_POOL_FULL = 5,     /* voxel-block pool exhausted                 */
    YAS_ERR_NUMERIC = 6,       /* NaN in the Gauss-Newton solve              */
    YAS_ERR_TRACK_LOST = 7,    /* |translation| of the frame step > limit    */
    YAS_ERR_MESH_OVERFLOW = 8, /* more triangles than the mesher's capacity  */
    YAS_ERR_STATE = 9,         /* call not valid in the handle's state       */
    YAS_ERR_COORD_RANGE = 10,  /* block coordinate outside the 21-bit range  */
    YAS_ERR_CAPACITY = 11,     /* caller buffer too small                    */
    YAS_ERR_TIMEOUT = 12,      /* a bounded device-side wait gave up         */
    YAS_ERR_IO = 13            /* a file could not be read or written        */
};

/* Human-readable name of a status code (static string). */
YAS_API const char *yas_status_string(int status);
/* Library version string, e.g. "yas-gb300 0.1.0 sm_103a". */
YAS_API const char *yas_version(void);

/* ---------------------------------------------------------------- PODs */
typedef struct yas_intrinsics {
    float fx, fy, cx, cy;
} yas_intrinsics;

typedef struct yas_pose {
    double m[12]; /* row-major [R | t] */
} yas_pose;

/* TSDF voxel storage formats.  All formats keep the reference's update rule
 * (running weighted average, weight + 1 capped at 255). */
enum yas_voxel_format {
    YAS_VOXEL_F32 = 0, /* float sdf + float weight, 8 B/voxel              */
    YAS_VOXEL_F16 = 1, /* fp16 sdf + u8 weight, 4 B/voxel; the spare byte  *
                        * keeps the fp16 rounding residual (1/256 ulp)    */
    YAS_VOXEL_S24 = 2, /* 24-bit fixed-point sdf (2^-22 step) + u8 weight, 4 B */
    YAS_VOXEL_S16 = 3  /* the reference's Voxel {short sdf; uchar wt;}, 4 B and *
                        * the same byte layout: sdf stored as (short)(s*32767) *
                        * truncated toward zero, read as q/32767 (PackFloat / *
                        * UnPackFloat, VoxelStructUtils.h:6-14)                */
};

typedef struct yas_map_config {
    int hash_slots;    /* open-addressing slots, power of two               */
    int max_blocks;    /* voxel-block pool capacity (8^3 voxels per block)  */
    float voxel_size;  /* metres                                            */
    float trunc_dist;  /* metres                                            */
    float depth_min;   /* fusion/visibility gate; reference: 0.1 m          */
    float depth_max;   /* fusion/visibility gate; reference: 3.0 m          */
    int voxel_format;  /* enum yas_voxel_format                             */
    int max_weight;    /* weight cap; reference: 255                        */
} yas_map_config;

/* Fills `cfg` with the reference's constants (depth 0.1..3.0 m, weight cap
 * 255) for the given grid; VoxelMap.cu:812-813,852-853. */
YAS_API int yas_map_config_default(yas_map_config *cfg, int hash_slots, int max_blocks,
                                   float voxel_size, float trunc_dist, int voxel_format);

/* ---------------------------------------------------------------- MapStruct
 * Replaces class MapStruct (RGBDFusion/include/VoxelMap.h:32-144). */
typedef struct yas_map yas_map;

/* MapStruct(K) + create(...) + Reset(): VoxelMap.h:35,38,45; VoxelMap.cu:46-93. */
YAS_API int yas_map_create(yas_map **out, const yas_map_config *cfg, const yas_intrinsics *K,
                           void *stream);
/* MapStruct::create(hashTableSize, bucketSize, voxelBlockSize, voxelSize,
 * truncationDist) argument form, VoxelMap.h:35 / VoxelMap.cu:60-81.  The slot
 * count becomes the power of two >= max(hashTableSize, 2*voxelBlockSize). */
YAS_API int yas_map_create_ref(yas_map **out, int hashTableSize, int bucketSize, int voxelBlockSize,
                               float voxelSize, float truncationDist, const yas_intrinsics *K,
                               void *stream);
/* MapStruct::Release(): VoxelMap.h:48 / VoxelMap.cu:104-136 (also frees the handle). */
YAS_API int yas_map_destroy(yas_map *map);
/* MapStruct::Reset(): VoxelMap.h:45 / VoxelMap.cu:46-58. */
YAS_API int yas_map_reset(yas_map *map);
/* MapStruct::Empty(): VoxelMap.h:46 / VoxelMap.cu:138-141 (no allocated block). */
YAS_API int yas_map_empty(yas_map *map, int *out_empty);
/* MapStruct::Fuse(GpuMat depth, SE3d Tcm): VoxelMap.h:61 / VoxelMap.cu:825-884.
 * depth: float metres, `on_device` = 1 for a device pointer, 0 for host. */
YAS_API int yas_map_fuse_depth(yas_map *map, const float *depth, int width, int height,
                               int pitch_bytes, int on_device, const yas_pose *Tcm);
/* MapStruct::CheckNumVisibleBlocks(cols, rows, Tcm): VoxelMap.h:59 / VoxelMap.cu:788-823. */
YAS_API int yas_map_check_visible(yas_map *map, int cols, int rows, const yas_pose *Tcm,
                                  unsigned *out_count);
/* MapStruct::GetNumVisibleBlocks(): VoxelMap.h:58 / VoxelMap.cu:201-206. */
YAS_API int yas_map_num_visible(yas_map *map, unsigned *out_count);
/* MapStruct::ResetNumVisibleBlocks / ResetVisibleBlocks: VoxelMap.cu:208-211,963-966
 * (the visible-block count drops to 0; the next raycast then starts from an
 * empty visible set until the next fusion or visibility check). */
YAS_API int yas_map_reset_visible(yas_map *map);
/* Number of allocated blocks (no reference counterpart; heap pointer). */
YAS_API int yas_map_num_allocated(yas_map *map, unsigned *out_count);
/* Sticky device error bits of the map (YAS_ERR_* as 1<<code), cleared on read. */
YAS_API int yas_map_take_errors(yas_map *map, unsigned *out_bits);
/* Copies every allocated block to host arrays: coords[3*i] = block x,y,z,
 * sdf/weight[512*i + z*64 + y*8 + x] (float).  Order: pool order. */
YAS_API int yas_map_export(yas_map *map, int *coords, float *sdf, float *weight, unsigned capacity,
                           unsigned *out_count);
/* Inserts blocks with given contents (the inverse of yas_map_export). */
YAS_API int yas_map_import(yas_map *map, const int *coords, const float *sdf, const float *weight,
                           unsigned count);
/* MapStruct::visibleTable contents as block coords (host), VoxelMap.h:127-128. */
YAS_API int yas_map_export_visible(yas_map *map, int *coords, unsigned capacity, unsigned *out_count);
/* MapStruct::GetPose / SetPose (host-side mTcw), VoxelMap.h:40-41 / VoxelMap.cu:12-22. */
YAS_API int yas_map_get_pose(yas_map *map, yas_pose *out);
YAS_API int yas_map_set_pose(yas_map *map, const yas_pose *Tcw);
/* MapStruct::SetActiveFlag / isActive, VoxelMap.h:73-74 / VoxelMap.cu:989-999. */
YAS_API int yas_map_set_active(yas_map *map, int flag);
YAS_API int yas_map_is_active(yas_map *map, int *out);
/* MapStruct::Hibernate / ReActivate (host swap of all device arrays),
 * VoxelMap.h:69-71 / VoxelMap.cu:894-954. */
YAS_API int yas_map_hibernate(yas_map *map);
YAS_API int yas_map_reactivate(yas_map *map);
YAS_API int yas_map_is_hibernated(yas_map *map, int *out);
/* Device-memory footprint in bytes (tables, pool, lists). */
YAS_API int yas_map_device_bytes(yas_map *map, size_t *out_bytes);
/* MapStruct::Reserve(hashTableSize, bucketSize, voxelBlockSize), VoxelMap.cu:479-515:
 * grows the table to >= hash_slots slots (power of two) and the pool to
 * >= max_blocks blocks; blocks keep their contents, the table is rebuilt. */
YAS_API int yas_map_reserve(yas_map *map, int hash_slots, int max_blocks);
/* MapStruct::SaveToFile / ReadFromFile (VoxelMap.h:65-66; empty stubs at
 * VoxelMap.cu:886-893): a binary submap file (144-byte header: magic
 * "YASSUBM1", version 3, voxel format, voxel size, truncation, depth gates,
 * weight cap, capacities, block count, pose; then int32 block coordinates; then
 * the voxels in the map's storage format).  Loading replaces the map's
 * contents and pose, grows it if needed, and needs the same voxel format and
 * size (YAS_ERR_BAD_ARG otherwise); the round trip is bit-exact. */
YAS_API int yas_map_save(yas_map *map, const char *path);
YAS_API int yas_map_load(yas_map *map, const char *path);
/* MapStruct::Swap(MapStruct*), VoxelMap.cu:173-199: the two maps exchange
 * their storage, grid configuration, intrinsics and hibernation state; each
 * handle keeps its pose and active flag, as in the reference. */
YAS_API int yas_map_swap(yas_map *map, yas_map *other);
/* MapStruct::Fuse(MapStruct *src), VoxelMap.cu:398-444 (System::FuseAllMapStruct,
 * System.cpp:73-93): fuses src into map using both maps' poses (yas_map_get_pose);
 * an empty map takes src's storage and pose.  src is left empty (the reference
 * releases it); destroy it with yas_map_destroy.  Same voxel size and format. */
YAS_API int yas_map_fuse_map(yas_map *map, yas_map *src);
/* No counterpart in the reference: removes the observation of one depth frame
 * at pose Tcm (the inverse of yas_map_fuse_depth's running average, exact
 * where that frame was fused and the weight stayed below the cap), for
 * re-integration after a pose correction. */
YAS_API int yas_map_defuse_depth(yas_map *map, const float *depth, int width, int height, int pitch_bytes,
                                 int on_device, const yas_pose *Tcm);

/* ---------------------------------------------------------------- RayTraceEngine
 * Replaces class RayTraceEngine (RGBDFusion/include/RayTraceEngine.h:11-49). */
typedef struct yas_raycaster yas_raycaster;

/* RayTraceEngine(w, h, K): RayTraceEngine.h:15 / RayTraceEngine.cu:11-29. */
YAS_API int yas_raycaster_create(yas_raycaster **out, int width, int height,
                                 const yas_intrinsics *K, void *stream);
YAS_API int yas_raycaster_destroy(yas_raycaster *rc);
/* RayTraceEngine::RayTrace(MapStruct*, Tcm): RayTraceEngine.h:16 / RayTraceEngine.cu:412-450. */
YAS_API int yas_raycaster_raycast(yas_raycaster *rc, yas_map *map, const yas_pose *Tcm);
/* RayTraceEngine::GetVMap(): device float4 vertex map (camera frame, w=+1 hit,
 * w=-1 miss), row pitch in bytes. RayTraceEngine.h:27 / RayTraceEngine.cu:452-455. */
YAS_API int yas_raycaster_vmap(yas_raycaster *rc, const float **dev_vmap, int *pitch_bytes);
/* MapStruct::GetRayTracingResultDepth(): VMapToDepth of the last raycast into
 * `depth` (float metres, 0 = miss), VoxelMap.cu:981-987 / ImageProc.cu:262-286. */
YAS_API int yas_raycaster_depth(yas_raycaster *rc, float *depth, int pitch_bytes, int on_device);
/* RayTraceEngine::GetNumVisibleBlock / GetNumRenderingBlocks: RayTraceEngine.h:25-26. */
YAS_API int yas_raycaster_num_visible(yas_raycaster *rc, unsigned *out);
YAS_API int yas_raycaster_num_rendering_blocks(yas_raycaster *rc, unsigned *out);
/* Copies the (W/8)x(H/8) z-range maps (near, far) to host float arrays. */
YAS_API int yas_raycaster_zrange(yas_raycaster *rc, float *znear, float *zfar);

/* ---------------------------------------------------------------- MeshEngine
 * Replaces class MeshEngine (RGBDFusion/include/MeshEngine.h:8-24). */
typedef struct yas_mesher yas_mesher;

/* MeshEngine(MaxNumTriangle): MeshEngine.h:12 / MeshEngine.cu:271-277. */
YAS_API int yas_mesher_create(yas_mesher **out, int max_triangles, void *stream);
YAS_API int yas_mesher_destroy(yas_mesher *me);
/* MeshEngine::Meshify(MapStruct*) device part: MeshEngine.h:13 / MeshEngine.cu:293-331.
 * Triangles are emitted block by block in pool order (deterministic for a given map). */
YAS_API int yas_mesher_meshify(yas_mesher *me, yas_map *map, unsigned *out_num_triangles);
/* D2H of the soup: 9 floats per triangle (3 vertices, submap metres) and the
 * face normal repeated per vertex, as MapStruct::mplPoint / mplNormal (N = 9 * count),
 * MeshEngine.cu:332-339. */
YAS_API int yas_mesher_copy(yas_mesher *me, float *points, float *normals, unsigned capacity_tris);
/* Per-triangle marching-cubes case index and global voxel position (for
 * topology checks): cases[i], cube_xyz[3*i]. */
YAS_API int yas_mesher_copy_cases(yas_mesher *me, int *cases, int *cube_xyz, unsigned capacity_tris);

/* ---------------------------------------------------------------- RGBDTracking
 * Replaces class RGBDTracking (RGBDFusion/include/RGBDTracking.h:9-107). */
typedef struct yas_tracker yas_tracker;

enum yas_track_mode { YAS_TRACK_RGB = 1, YAS_TRACK_ICP = 2, YAS_TRACK_RGBD = 3 };

/* RGBDTracking(w, h, K, bRGB, bIcp): RGBDTracking.h:13 / RGBDTracking.cu:5-64.
 * K: row-major 3x3 double.  num_levels <= 5 (reference: 5); iterations[l] is
 * the GN iteration count at level l (reference: {10,5,3,3,3}). */
YAS_API int yas_tracker_create(yas_tracker **out, int width, int height, const double *K,
                               int num_levels, const int *iterations, int mode, void *stream);
YAS_API int yas_tracker_destroy(yas_tracker *tr);
/* SetReferenceImage / SetTrackingImage (CV_8U gray): RGBDTracking.h:17,20 / .cu:66-116. */
YAS_API int yas_tracker_set_reference_image(yas_tracker *tr, const uint8_t *gray, int pitch_bytes,
                                            int on_device);
YAS_API int yas_tracker_set_tracking_image(yas_tracker *tr, const uint8_t *gray, int pitch_bytes,
                                           int on_device);
/* SetReferenceDepth / SetTrackingDepth (CV_32F metres): RGBDTracking.h:18,21 / .cu:80-138. */
YAS_API int yas_tracker_set_reference_depth(yas_tracker *tr, const float *depth, int pitch_bytes,
                                            int on_device);
YAS_API int yas_tracker_set_tracking_depth(yas_tracker *tr, const float *depth, int pitch_bytes,
                                           int on_device);
/* SetReferenceModel(GpuMat vmap): RGBDTracking.h:23 / RGBDTracking.cu:140-150.
 * vmap: device float4 (w=+1 valid). */
YAS_API int yas_tracker_set_reference_model(yas_tracker *tr, const float *dev_vmap, int pitch_bytes);
/* GetTransform(init, bSwapBuffer): RGBDTracking.h:27 / RGBDTracking.cu:152-214. */
YAS_API int yas_tracker_get_transform(yas_tracker *tr, const yas_pose *init, int swap_buffer,
                                      yas_pose *out);
/* No counterpart in the reference: 1 (default) runs GetTransform's whole
 * coarse-to-fine schedule as one cooperative launch; 0 launches the two
 * pixel passes of every iteration separately.  Results agree within the
 * rounding of a different summation order. */
YAS_API int yas_tracker_set_schedule(yas_tracker *tr, int fused);
/* How the Gauss-Newton sums are totalled across the GPU.  1 (default):
 * compensated FP32 (TwoSum) partial sums, totals kept as double-float pairs
 * (FP64 totals in the per-iteration passes).  0: plain FP32 sums in the same
 * order, the reference's arithmetic (WarpReduceSum / BlockReduceSum and
 * cv::cuda::reduce in FP32, TrackingUtils.h:8-58, RGBDTracking.cu:253-286),
 * for precision comparisons.  The solve is double-float (48 significant
 * bits) either way.  Takes effect at the next GetTransform, captured graphs
 * included. */
YAS_API int yas_tracker_set_reduction(yas_tracker *tr, int compensated);
/* Checks the fused GN schedule's bounded waits (no counterpart in the
 * reference).  Runs the schedule on the tracker's current images as a launch
 * whose descriptor names two CTAs but starts one, so the waits for the missing
 * CTA's partial sums run out: after about 1 s the schedule records a timeout
 * and ends.  *out_status receives what the schedule reports (YAS_ERR_TIMEOUT
 * when the limit works).  The tracker stays usable; its next GetTransform
 * starts from a reset state.  Takes about one second. */
YAS_API int yas_tracker_check_wait_limit(yas_tracker *tr, int *out_status);
/* Checks the division the device solve uses for its pivots (no counterpart
 * in the reference: the reference divides on the host in Eigen).
 * out[i] = a[i] / x[i] computed on the device as the solve computes it: the
 * operands rounded to double-float (FP32 pairs), the approximate FP32
 * reciprocal of the divisor's high part refined by one Newton-Raphson step
 * and multiplied by the dividend, for 1e-30 < |x| < 1e30; an FP64 division of the rounded
 * operands outside that range.  Host arrays of n doubles, 0 < n <= 1 << 20;
 * waits for the result. */
YAS_API int yas_check_div_seeded(const double *a, const double *x, double *out, int n);
/* SwapFrameBuffer / IsTrackingGood: RGBDTracking.h:28,15 / RGBDTracking.cu:294-303,551-554. */
YAS_API int yas_tracker_swap_frame_buffer(yas_tracker *tr);
YAS_API int yas_tracker_is_good(yas_tracker *tr, int *out);
/* One Gauss-Newton linearisation at pose T on `level` (ComputeSingleStep*,
 * RGBDTracking.cu:225-292, 408-441, 521-545): H (36, row-major), b (6), and
 * stats[4] = {sum r^2 used for the error, residual count, rgb sigma, icp count}. */
YAS_API int yas_tracker_compute_step(yas_tracker *tr, int level, const yas_pose *T, double *H,
                                     double *b, double *stats);
/* The last Gauss-Newton solve of the tracker's last GetTransform or
 * compute_step (no counterpart in the reference; for inspection and tests):
 * the combined system H (36, row-major) and b (6) it solved, the update x
 * (6: translation then rotation, LDLT(H).solve(b)) and the estimate after
 * it (exp(x) * the estimate before).  Any pointer may be null; waits for the
 * tracker's stream. */
YAS_API int yas_tracker_last_solve(yas_tracker *tr, double *H, double *b, double *update, yas_pose *estimate);
/* Device pointers of pyramid level buffers (for inspection/tests).
 * which: 0 cur intensity, 1 cur gx, 2 cur gy, 3 cur inv-depth, 4 cur vmap,
 * 5 cur nmap, 6 ref intensity, 7 ref inv-depth, 8 ref vmap, 9 ref nmap. */
YAS_API int yas_tracker_level_buffer(yas_tracker *tr, int level, int which, const void **dev_ptr,
                                     int *width, int *height, int *pitch_bytes);

/* One pyramid level of the tracker's inputs, as device pointers to dense
 * row-major images of width x height (no padding).  vmap/nmap are float4
 * (x, y, z, w) with w > 0 for valid entries. */
typedef struct yas_gn_level {
    int width, height;
    float fx, fy, cx, cy;       /* intrinsics of this level                   */
    const float *ref_intensity; /* reference frame intensity                  */
    const float *ref_inv_depth; /* reference frame inverse depth (0 = none)   */
    const float *ref_vmap;      /* reference model vertices (float4)          */
    const float *ref_nmap;      /* reference model normals (float4)           */
    const float *cur_intensity; /* current frame intensity                    */
    const float *cur_gx;        /* current frame intensity gradient x         */
    const float *cur_gy;        /* current frame intensity gradient y         */
    const float *cur_vmap;      /* current frame vertices (float4)            */
    const float *cur_nmap;      /* current frame normals (float4)             */
} yas_gn_level;

/* No counterpart in the reference.  One Gauss-Newton linearisation at pose T
 * (what yas_tracker_compute_step computes: H, b and the statistics) for
 * callers that must not allocate device memory: a host that owns the whole
 * device-memory budget of the process, or code that runs where an allocation
 * would synchronise the device or is not allowed (inside a real-time frame
 * callback).  It allocates nothing: its scratch (per-pixel residuals, per-CTA
 * partial sums, tickets and the solver state) is a fixed array of about
 * 5.3 MB in the library's static device memory, present on every device that
 * loads the library until the process exits.
 * Limits: width * height <= 640 * 480 and width, height >= 4; larger levels
 * return YAS_ERR_CAPACITY before any work is enqueued.  mode: enum
 * yas_track_mode.  dev_out (device, 46 doubles): H row-major (36), b (6),
 * stats (4) as yas_tracker_compute_step.  The sums are always the compensated
 * reduction (TwoSum FP32 partial sums, FP64 totals), whatever
 * yas_tracker_set_reduction chose for any tracker; with that reduction the
 * result is bit-identical to yas_tracker_compute_step's for the same maps.
 * The first call on a device, and the first after the device's context
 * changes (e.g. after cudaDeviceReset), resolves the scratch address (no
 * allocation); make that call before capturing a stream.  All calls share the
 * one scratch array, which keeps the last call's contents (the call clears
 * what must start at zero), so calls whose GPU work overlaps (other streams,
 * other host threads) race and must be serialised by the caller; the call
 * itself only enqueues work on `stream` (NULL: legacy default stream). */
YAS_API int yas_gn_linearise_static(const yas_gn_level *level, const yas_pose *T, int mode, double *dev_out,
                                    void *stream);

/* ---------------------------------------------------------------- copies
 * No counterpart in the reference (which downloads cv::cuda::GpuMat): copies a
 * pitched 2-D region, `height` rows of `width_bytes`, from host or device
 * memory into host memory and waits for it, so host code can read the
 * library's device buffers without linking the CUDA runtime itself. */
YAS_API int yas_copy_to_host(void *dst, int dst_pitch, const void *src, int src_pitch, int width_bytes, int height);

/* ---------------------------------------------------------------- ImageProc free functions
 * RGBDFusion/include/ImageProc.h:8-24.  Device images (cv::cuda::GpuMat):
 * pointer, size, row pitch in bytes; float, or float4 for vertex / normal
 * maps.  Asynchronous on `stream`; outputs are written as the reference
 * kernels write them (pixels the reference leaves untouched stay as they are). */
/* PyrDownDepth (ImageProc.cu:166-187): dst(x, y) = src(2x, 2y) except dst's last row and column. */
YAS_API int yas_pyr_down_depth(const float *src, int src_w, int src_h, int src_pitch, float *dst, int dst_w,
                               int dst_h, int dst_pitch, void *stream);
/* DepthToInvDepth (ImageProc.cu:141-164): 1/z for 0.2 < z < 8 m, else 0. */
YAS_API int yas_depth_to_inv_depth(const float *depth, int w, int h, int pitch, float *inv_depth, int inv_pitch,
                                   void *stream);
/* ComputeVertexMap (ImageProc.cu:189-220): from inverse depth; w = -1 where invalid. */
YAS_API int yas_compute_vertex_map(const float *inv_depth, int w, int h, int pitch, float *vmap, int vmap_pitch,
                                   float invfx, float invfy, float cx, float cy, float cut_off, void *stream);
/* ComputeNormalMap (ImageProc.cu:222-260): normalize((v(x,y+1) - v) x (v(x+1,y) - v)). */
YAS_API int yas_compute_normal_map(const float *vmap, int w, int h, int pitch, float *nmap, int nmap_pitch,
                                   void *stream);
/* ComputeImageGradientCentralDifference (ImageProc.cu:7-40): 0.5 central differences, 0 on the border. */
YAS_API int yas_image_gradient(const float *image, int w, int h, int pitch, float *gx, float *gy, int grad_pitch,
                               void *stream);
/* TransformReferencePoint (ImageProc.cu:42-78): points of an inverse-depth image
 * moved by T: (R K^-1) (x, y, 1) z + t, R K^-1 formed in FP64 and rounded to FP32.
 * K: row-major 3x3 double. */
YAS_API int yas_transform_reference_point(const float *inv_depth, int w, int h, int pitch, float *vmap,
                                          int vmap_pitch, const double *K, const yas_pose *T, void *stream);
/* VMapToDepth (ImageProc.cu:262-286): z of valid vertices, else 0. */
YAS_API int yas_vmap_to_depth(const float *vmap, int w, int h, int pitch, float *depth, int depth_pitch,
                              void *stream);

/* ---------------------------------------------------------------- shading
 * RenderScene(vmap, nmap, image), ImageProc.cu:128-139 (ImageProc.h:17): Phong
 * shading of a device vertex/normal map (float4, camera frame, the same row
 * pitch) into RGBA8 for display, headless (no GL).  light: 3 floats in the
 * camera frame (NULL: the reference's (5, 5, 5)).  rgba: device memory
 * (on_device = 1) or host memory (0, copied back before return). */
YAS_API int yas_render_scene(const float *dev_vmap, const float *dev_nmap, int width, int height, int pitch_bytes,
                             const float *light, uint8_t *rgba, int out_pitch_bytes, int on_device, void *stream);

/* ---------------------------------------------------------------- mesh canvas
 * The viewer's mesh drawing (FullSystem/src/MapDrawer.cpp:159-234 with the GLSL
 * program of :13-58), headless: submap meshes are shaded per vertex as the
 * vertex shader does (light (5, 5, 5), viewer at the submap origin, in submap
 * coordinates) and rasterised with a z-buffer into a device image: placed by
 * Tmw (submap -> world, MapStruct::GetPose) and Tcw (world -> camera), pinhole
 * intrinsics with pixel centres at integer coordinates, perspective-correct
 * Gouraud interpolation, white background, triangles with a vertex nearer
 * than 5 cm left out.  Meshes drawn after one another share the z-buffer. */
typedef struct yas_canvas yas_canvas;
YAS_API int yas_canvas_create(yas_canvas **out, int width, int height, const yas_intrinsics *K, void *stream);
YAS_API int yas_canvas_destroy(yas_canvas *c);
/* Empties the z-buffer (the image reads white). */
YAS_API int yas_canvas_clear(yas_canvas *c);
/* A triangle soup as MeshEngine writes it: 9 floats per triangle (submap
 * metres) and the normal per vertex; host (on_device = 0) or device memory. */
YAS_API int yas_canvas_draw_triangles(yas_canvas *c, const float *points, const float *normals, unsigned n_tris,
                                      int on_device, const yas_pose *Tmw, const yas_pose *Tcw);
/* The mesher's last mesh, from its device buffers (no copy to the host). */
YAS_API int yas_canvas_draw_mesh(yas_canvas *c, yas_mesher *me, const yas_pose *Tmw, const yas_pose *Tcw);
/* RGBA8 image and depth (metres, 0 where empty) of the z-buffer; either may be
 * NULL; host (on_device = 0, copied back before return) or device memory. */
YAS_API int yas_canvas_read(yas_canvas *c, uint8_t *rgba, int rgba_pitch, float *depth, int depth_pitch,
                            int on_device);

/* ---------------------------------------------------------------- session
 * One SLAM session: a submap, a raycaster and a tracker whose per-frame dense
 * work (Tracking::TrackRGBD + Tracking::StereoInitialization dense calls,
 * FullSystem/src/Tracking.cpp:139-155,162-197; System::TrackRGBD colour and
 * depth conversion, FullSystem/src/System.cpp:43-65) runs as one captured
 * CUDA graph with no host round trip inside the frame. */
typedef struct yas_session yas_session;

typedef struct yas_session_config {
    int width, height;
    yas_intrinsics K;
    yas_map_config map;
    int num_levels;        /* pyramid levels (<= 5)                          */
    int iterations[5];     /* GN iterations per level, finest first          */
    int mode;              /* enum yas_track_mode                            */
    float depth_scale;     /* metres per depth unit (u16 mm: 0.001)          */
    float max_step_translation; /* frame-step rejection, reference 0.1 m     */
    int use_graph;         /* 1: capture the frame into a CUDA graph          */
    int fused_schedule;    /* 1: all GN iterations in one cooperative launch  */
} yas_session_config;

YAS_API int yas_session_config_default(yas_session_config *cfg, int width, int height,
                                       const yas_intrinsics *K, int hash_slots, int max_blocks,
                                       float voxel_size, float trunc_dist, int voxel_format);
YAS_API int yas_session_create(yas_session **out, const yas_session_config *cfg, void *stream);
YAS_API int yas_session_destroy(yas_session *s);
/* Enqueues one frame (RGB u8 interleaved w*h*3, depth u16 w*h) without waiting.
 * Inputs (host or device) must stay valid and unchanged until yas_session_wait
 * returns.  A tracked frame's graph reads 16-byte-aligned device memory of the
 * session's GPU or pinned host memory itself, beside the raycast; other inputs
 * are first copied on the session stream.  Either way the frame reads exactly
 * w*h*3 and w*h*2 bytes. */
YAS_API int yas_session_submit(yas_session *s, const uint8_t *rgb, const uint16_t *depth,
                               int on_device);
/* Waits for the last submitted frame; returns its map pose Tcm and frame status
 * (YAS_OK, YAS_ERR_TRACK_LOST, YAS_ERR_NUMERIC, ...). */
YAS_API int yas_session_wait(yas_session *s, yas_pose *out_Tcm, int *out_frame_status);
/* submit + wait. */
YAS_API int yas_session_process_frame(yas_session *s, const uint8_t *rgb, const uint16_t *depth,
                                      int on_device, yas_pose *out_Tcm, int *out_frame_status);
YAS_API int yas_session_map(yas_session *s, yas_map **out);
YAS_API int yas_session_tracker(yas_session *s, yas_tracker **out);
YAS_API int yas_session_raycaster(yas_session *s, yas_raycaster **out);
YAS_API int yas_session_frame_count(yas_session *s, int *out);
/* The submap switch of Tracking::CreateNewKeyFrame (Tracking.cpp:700-718):
 * the current submap is deactivated and handed to the caller (who owns it:
 * yas_map_fuse_map or yas_map_destroy); a new empty submap with the same
 * configuration, posed at the current camera's world pose (previous submap
 * pose * Tcm), continues the session, and Tcm restarts at the identity. */
YAS_API int yas_session_new_submap(yas_session *s, yas_map **out_previous);
/* Device pointer of the session's float depth (metres) of the last frame. */
YAS_API int yas_session_depth(yas_session *s, const float **dev_depth, int *pitch_bytes);
/* Number of kernels the last frame launched (graph nodes of kind kernel). */
YAS_API int yas_session_kernels_per_frame(yas_session *s, int *out);

/* Stream of a handle (cudaStream_t as void*), for event timing by callers. */
YAS_API void *yas_session_stream(yas_session *s);
/* Runs one tracked frame eagerly with a CUDA event before every launch group
 * and returns the device time of each group: stage_ids[i] is 0 image
 * pyramid, 1 depth pyramid, 2 z-range, 3 ray march, 4 model pyramid, 5 GN
 * init, 10+l / 20+l GN pass A / B at level l, 6 frame finalize, 7 block
 * allocation, 8 visibility, 9 integration; stage_ms[i] its duration. */
YAS_API int yas_session_profile_frame(yas_session *s, const uint8_t *rgb, const uint16_t *depth, int on_device,
                                      int *stage_ids, float *stage_ms, int capacity, int *out_count);

/* ---------------------------------------------------------------- batched submaps
 * No counterpart in the reference, which tracks and fuses one keyframe submap
 * at a time (FullSystem/src/Tracking.cpp:162-197).  A batch steps many
 * sessions together: keyframe submaps of any resolution and voxel size.  One
 * step runs one frame of every active session as a single CUDA graph launch.
 * The graph holds:
 *   - each session's pyramids, raycast and model pyramid, as parallel branches;
 *   - one persistent cooperative Gauss-Newton launch over all their pyramid
 *     levels (split in two only if the CTAs exceed what is co-resident);
 *   - each session's pose update and fusion (allocation, visibility,
 *     integration).
 * A graph is captured once per combination of the sessions' states (inactive,
 * initialising, tracked on either frame-buffer parity) and then reused.  The
 * sessions stay owned by the caller, who must not drive them by other calls
 * while the batch steps them. */
typedef struct yas_batch yas_batch;

typedef struct yas_batch_tuning {
    int march_warps_x;     /* ray march: 1, 2, 4: one thread per pixel, CTA tiles of
                            * 8x16, 16x8, 32x4 pixels; 0: persistent warps taking 8x4
                            * tiles from a queue (the vertex map is the same for all) */
    int integrate_ctas;    /* CTAs of the integration grid, 256 threads each          */
    int gn_pixels_per_cta; /* batched GN: 0 splits the co-resident 1024-thread CTAs
                            * over the step's sessions in proportion to their pixels;
                            * > 0: one CTA per this many level-0 pixels (1..16 per
                            * session), which fixes each session's summation order, so
                            * its results do not depend on the rest of the batch      */
    int gn_per_session;    /* 1: each session's GN schedule is its own cooperative
                            * launch in the session's branch of the graph (sessions
                            * overlap their halves with other sessions' GN); 0: one
                            * launch for every session of the step (split only if
                            * its CTAs exceed what is co-resident); same results    */
} yas_batch_tuning;

/* Defaults: 2, 1216 (152 x 8), 0, 1. */
YAS_API int yas_batch_tuning_default(yas_batch_tuning *t);
YAS_API int yas_batch_create(yas_batch **out, yas_session *const *sessions, int count, void *stream);
YAS_API int yas_batch_destroy(yas_batch *b);
YAS_API int yas_batch_set_tuning(yas_batch *b, const yas_batch_tuning *t);
YAS_API int yas_batch_get_tuning(yas_batch *b, yas_batch_tuning *out);
/* Enqueues one frame of every session i with active[i] != 0 (active NULL: all).
 * rgb[i] / depth[i] as for yas_session_submit (host memory must stay valid
 * until yas_batch_wait returns).  Does not wait. */
YAS_API int yas_batch_step(yas_batch *b, const uint8_t *const *rgb, const uint16_t *const *depth,
                           const int *active, int on_device);
/* Waits for the last step.  For every session it ran: its map pose and frame
 * status (other entries are left as they are; either array may be NULL).
 * out_ms (may be NULL): device time of the step, input copies included. */
YAS_API int yas_batch_wait(yas_batch *b, yas_pose *out_Tcm, int *out_status, float *out_ms);
/* Kernel nodes of the last step's graph. */
YAS_API int yas_batch_kernels_per_step(yas_batch *b, int *out);
/* The launch-shape autotuner.  It copies every session's configuration into
 * scratch sessions and runs them through the first `frames` (>= 3) frames of
 * each session: rgb[i] / depth[i] hold that many consecutive frames.  Each
 * knob (GN share, march CTA shape, integration grid) is tried in turn over a
 * few candidate values (GN share, GN launches per session or per step, march
 * CTA shape, integration grid), the others held, each candidate timed by the median
 * device time of its tracked steps over three passes.  A value replaces the
 * current one only if it is more than 3 % faster, and the final choice must
 * beat the starting tuning by that margin again when both are re-measured.
 * It is applied to the batch and written to *out (may be NULL).  The batch's
 * own sessions are not touched. */
YAS_API int yas_batch_autotune(yas_batch *b, const uint8_t *const *rgb, const uint16_t *const *depth, int frames,
                               int on_device, yas_batch_tuning *out);

/* ---------------------------------------------------------------- served sessions
 * No counterpart in the reference, which runs one session per process
 * (FullSystem/src/System.cpp:43-65).  A request server runs the frames of many
 * sessions with continuous batching: frames submitted while others are on the
 * GPU join the next batch as soon as their session has no frame in flight;
 * each batch runs its sessions' per-frame work on their own streams and all
 * their Gauss-Newton schedules in one launch.  Sessions are admitted by free
 * HBM.  A session's results do not depend on which other sessions share its
 * batches. */
typedef struct yas_server yas_server;

typedef struct yas_server_config {
    int max_sessions;         /* live sessions at most                               */
    size_t hbm_reserve_bytes; /* admission: free HBM - session footprint >= this    */
    int ring_frames;          /* queued frames per session (pinned input ring)      */
    int gn_per_session;       /* 1: a taken frame runs its own Gauss-Newton launch  *
                               * (a fixed CTA share) on its session's stream at   *
                               * once; 0: sessions whose first half is queued     *
                               * gather into one batched launch                   */
    int gn_pixels_per_cta;    /* gn_per_session: a session's GN share is one CTA per *
                               * this many level-0 pixels, at most 32 CTAs (0: the *
                               * default, 16384)                                   */
} yas_server_config;

typedef struct yas_served_result {
    int session;       /* session id                                           */
    int status;        /* frame status, as yas_session_wait                    */
    long long frame;   /* frame number within the session (0 = initialising)   */
    double latency_ms; /* submission to completion                             */
    yas_pose Tcm;      /* map pose after the frame                             */
} yas_served_result;

typedef struct yas_server_stats {
    long long frames;  /* completed frames since the last reset                */
    long long batches; /* batched GN launches                                  */
    double mean_batch; /* tracked frames per batch                             */
    double p50_ms, p99_ms, max_ms; /* per-frame latency                        */
    double fps;        /* completed frames / (last completion - first submission) */
} yas_server_stats;

/* Defaults: 64 sessions, 4 GiB reserve, 4 queued frames per session, GN per
 * session. */
YAS_API int yas_server_config_default(yas_server_config *cfg);
/* Starts the server's worker thread on the current device. */
YAS_API int yas_server_create(yas_server **out, const yas_server_config *cfg);
/* Stops the worker, waits for the GPU and frees every session. */
YAS_API int yas_server_destroy(yas_server *srv);
/* Admits a session (YAS_ERR_OOM: its footprint does not fit the free HBM minus
 * the reserve; YAS_ERR_CAPACITY: max_sessions live). */
YAS_API int yas_server_open_session(yas_server *srv, const yas_session_config *cfg, int *out_id);
/* Eviction (MapStruct::Hibernate / ReActivate, VoxelMap.cu:894-954): suspend
 * waits for the session's frame in flight and moves its map to host memory,
 * freeing its HBM; frames submitted meanwhile stay queued.  Resume is admitted
 * like a new session (YAS_ERR_OOM if the map does not fit the free HBM minus
 * the reserve) and brings the map back. */
YAS_API int yas_server_suspend_session(yas_server *srv, int id);
YAS_API int yas_server_resume_session(yas_server *srv, int id);
/* Drops the session's queued frames, waits for its frame in flight, frees it. */
YAS_API int yas_server_close_session(yas_server *srv, int id);
/* Queues one frame (host RGB u8 interleaved, depth u16; copied before the call
 * returns).  YAS_ERR_CAPACITY: the session's input ring is full. */
YAS_API int yas_server_submit(yas_server *srv, int id, const uint8_t *rgb, const uint16_t *depth);
/* Takes up to `capacity` completed results, oldest first. */
YAS_API int yas_server_poll(yas_server *srv, yas_served_result *out, int capacity, int *out_count);
/* Waits until no frame is queued or in flight (YAS_ERR_TIMEOUT after timeout_s). */
YAS_API int yas_server_drain(yas_server *srv, double timeout_s);
YAS_API int yas_server_get_stats(yas_server *srv, yas_server_stats *out);
YAS_API int yas_server_reset_stats(yas_server *srv);

#ifdef __cplusplus
}
#endif
#endif /* YAS_H */
