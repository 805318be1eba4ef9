// session.cu — one SLAM session's per-frame dense pipeline as a CUDA graph.
//
// Reference flow (paths relative to the reference project root):
//   first frame   FullSystem/src/Tracking.cpp:139-155 (StereoInitialization):
//                 SetReferenceImage, SetReferenceDepth, Fuse(depth, identity).
//   later frames  Tracking.cpp:162-197 (TrackRGBD): RayTrace(Tcm_last) ->
//                 SetReferenceModel(vmap) -> SetTrackingImage/Depth ->
//                 DT = GetTransform(identity, swap) -> reject |t(DT)| > 0.1 m ->
//                 Tcm = Tcm_last * DT^-1 -> Fuse(depth, Tcm).
//   colour/depth  FullSystem/src/System.cpp:43-65 (RGB -> gray, u16 -> metres).
//
// GB300 design: the whole frame (preprocessing, raycast, model pyramid, every
// Gauss-Newton iteration with its device-side solve, the frame-step check,
// the pose update, block allocation, visibility and integration) is one
// captured graph; the only host traffic per frame is the input upload before
// the graph and one 200-byte frame record copied back at its end.  The frame
// step check and pose composition run on the device, and fusion kernels read
// a skip flag, so a rejected frame changes nothing.  The raycast reuses the
// visible-block list of the previous fusion, which was built at exactly the
// pose the raycast uses, so its z-range tiles are filled right after that
// fusion's visibility pass, beside its integration, and the next frame starts
// with the march.  Two graphs alternate because the reference and
// current pyramids swap roles every frame (RGBDTracking::SwapFrameBuffer,
// RGBDTracking.cu:294-303).
// Deliberate difference: a NaN in the solve skips fusion and reports
// YAS_ERR_NUMERIC (the reference fuses at the previous pose).
#include <cstring>

#include "yas_session.h"

namespace yas {

struct __align__(16) FrameState {
    PosePair pp;      // current Tcm in float (T) and its inverse (Tinv)
    double Tcm[12];   // current Tcm, row-major [R|t]
    double dt[12];    // last frame step DT (current <- previous)
    int skip;         // 1: fusion kernels return immediately
    int status;       // yas_status of the last frame
    int frame;        // frames processed
    int pad;
};

// Float pose pair of fs->Tcm, one lane per entry (lanes 0..11).  The inverse
// translation is rounded once per operation, in the order of the host's
// pose_inverse (built without contraction), so a frame fused by the session
// and the same frame given to yas_map_fuse_depth / yas_map_defuse_depth at the
// returned pose use the same float pose.
__device__ void publish_pose(FrameState *fs, int lane) {
    const double *T = fs->Tcm;
    if (lane < 12) {
        const int i = lane / 4, j = lane % 4;
        if (j < 3) {
            fs->pp.T.r[i * 3 + j] = (float)T[i * 4 + j];
            fs->pp.Tinv.r[i * 3 + j] = (float)T[j * 4 + i];
        } else {
            fs->pp.T.t[i] = (float)T[i * 4 + 3];
            const double s = __dadd_rn(__dadd_rn(__dmul_rn(T[0 * 4 + i], T[3]), __dmul_rn(T[1 * 4 + i], T[7])),
                                       __dmul_rn(T[2 * 4 + i], T[11]));
            fs->pp.Tinv.t[i] = (float)(-s);
        }
    }
}

__global__ void frame_begin_kernel(FrameState *fs, Pose64 init, MapHeader *hdr) {
    const int lane = threadIdx.x;
    if (lane < 12) {
        const int i = lane / 4, j = lane % 4;
        fs->Tcm[lane] = j < 3 ? init.r[i * 3 + j] : init.t[i];
        fs->dt[lane] = (lane % 5 == 0) ? 1.0 : 0.0;
    }
    __syncwarp();
    publish_pose(fs, lane);
    if (lane == 0) {
        fs->skip = 0;
        fs->status = YAS_OK;
        fs->frame = 1;
        hdr->n_visible = 0;
    }
}

// The frame state into the host's pinned copy (mapped memory; the host reads
// it once the stream is synchronised), one warp.
__device__ __forceinline__ void frame_state_to_host(const FrameState *fs, FrameState *host, int lane) {
    __syncwarp();
    const unsigned *src = reinterpret_cast<const unsigned *>(fs);
    unsigned *dst = reinterpret_cast<unsigned *>(host);
    for (int i = lane; i < (int)(sizeof(FrameState) / 4); i += 32) dst[i] = src[i];
}

// Frame-step check and pose composition: Tcm <- Tcm * DT^-1 (Tracking.cpp:178-187),
// one warp, one lane per matrix entry (FP64 issues at the same cost for one or
// 32 active lanes on GB300); the result also goes to the host's copy.
__global__ void frame_finalize_kernel(FrameState *fs, const GNState *st, float max_t, MapHeader *hdr,
                                      FrameState *host) {
    release_dependents();
    const int lane = threadIdx.x;
    __shared__ double Di[12], A[12];
    __shared__ int ok;
    const double *D = st->best;
    if (lane == 0) {
        fs->frame += 1;
        // |t| > max_t, compared squared (no FP64 square root)
        const double tn2 = D[3] * D[3] + D[7] * D[7] + D[11] * D[11];
        ok = 1;
        if (st->failed) {
            fs->status = st->failed == kFailTimeout ? YAS_ERR_TIMEOUT : YAS_ERR_NUMERIC;
            fs->skip = 1;
            ok = 0;
        } else if (!(tn2 <= (double)max_t * (double)max_t)) {
            fs->status = YAS_ERR_TRACK_LOST;
            fs->skip = 1;
            ok = 0;
        }
    }
    __syncwarp();
    if (!st->failed && lane < 12) fs->dt[lane] = D[lane];
    if (!ok) {
        frame_state_to_host(fs, host, lane);
        return;
    }
    if (lane < 12) {
        // DT^-1 = [R^T | -R^T t]
        const int i = lane / 4, j = lane % 4;
        Di[lane] = j < 3 ? D[j * 4 + i] : -((D[0 * 4 + i] * D[3] + D[1 * 4 + i] * D[7]) + D[2 * 4 + i] * D[11]);
        A[lane] = fs->Tcm[lane];
    }
    __syncwarp();
    if (lane < 12) {
        const int i = lane / 4, j = lane % 4;
        double o = (A[i * 4 + 0] * Di[0 * 4 + j] + A[i * 4 + 1] * Di[1 * 4 + j]) + A[i * 4 + 2] * Di[2 * 4 + j];
        if (j == 3) o += A[i * 4 + 3];
        fs->Tcm[lane] = o;
    }
    __syncwarp();
    publish_pose(fs, lane);
    if (lane == 0) {
        fs->skip = 0;
        fs->status = YAS_OK;
        hdr->n_visible = 0;
    }
    frame_state_to_host(fs, host, lane);
}

// A frame's input copy, the first node of a captured frame's frame branch: the
// caller's rgb and depth (device memory, or pinned host memory the device
// maps) into the session's buffers, 16 bytes per thread.  Its sources are set
// on the node before every launch, so the copy runs beside the raycast branch
// instead of ahead of the whole frame.  n_rgb = n_depth = 0 (the copies ran on
// the stream before the launch) makes it return at once.
__global__ void __launch_bounds__(256) input_copy_kernel(const uint4 *__restrict__ rgb,
                                                         const uint4 *__restrict__ depth, uint4 *__restrict__ d_rgb,
                                                         uint4 *__restrict__ d_depth, unsigned n_rgb,
                                                         unsigned n_depth) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_rgb)
        d_rgb[i] = rgb[i];
    else if (i - n_rgb < n_depth)
        d_depth[i - n_rgb] = depth[i - n_rgb];
}

}  // namespace yas

using namespace yas;

struct yas_session {
    yas_session_config cfg;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    yas_map *map = nullptr;
    yas_raycaster *rc = nullptr;
    // z-range tiles of the next frame's raycast (the session's own, so calls on
    // its raycaster between frames leave them alone): filled after each
    // frame's visibility pass, which is at the pose the next raycast uses
    RaycastBuffers zt = {};
    yas_tracker *tr = nullptr;
    uint8_t *d_rgb = nullptr;
    uint16_t *d_depth = nullptr;
    float *d_depth_m = nullptr;
    FrameState *fs = nullptr;
    FrameState *fs_host = nullptr;
    FrameState *fs_host_dev = nullptr;  // fs_host as the device maps it
    int frames = 0;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    // the graphs exec[] came from, kept for their input-copy nodes, which are
    // updated before every launch (null node: the copies run on the stream)
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphNode_t input_node[2] = {nullptr, nullptr};
    const void *input_src[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // the nodes' current sources
    bool capture_input = false;  // capturing exec[]: the frame branch starts with the input copy
    int device = 0;
    cudaGraphExec_t pre_exec[2] = {nullptr, nullptr};  // served frames: up to the GN schedule
    cudaGraphExec_t post_exec = nullptr;               // served frames: after it
    // the map's device arrays when the graphs were captured: growth, fusion
    // into this map and hibernation move them, and the graphs are captured again
    const void *graph_arrays[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // second stream of a tracked frame: the raycast branch runs beside the
    // pyramids of the new frame (fork/join events, captured as graph branches)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int kernels_per_frame = 0;
    LaunchShape shape;
    Cam cam;
    // profiling: events recorded between launches of an eager frame
    std::vector<cudaEvent_t> prof_events;
    std::vector<int> prof_ids;
    bool profiling = false;
};

// Records an event tagged `id` before the next launch (profiling only).
static void prof_mark(void *ctx, int id) {
    yas_session *s = static_cast<yas_session *>(ctx);
    if (!s->profiling) return;
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, s->stream);
    s->prof_events.push_back(e);
    s->prof_ids.push_back(id);
}

// Stage ids of the profiling marks (pass A / B of level l are 10+l / 20+l).
enum { kStImage = 0, kStDepth = 1, kStZrange = 2, kStMarch = 3, kStModel = 4, kStGnInit = 5,
       kStFinalize = 6, kStAllocate = 7, kStVisible = 8, kStIntegrate = 9, kStEnd = 99 };

// The next raycast's z-range tiles (RayTraceEngine.cu:58-264) from the map's
// visible list and the frame pose pair: both are final once a frame's
// visibility pass has run, and nothing changes them before the next frame's
// march.
static void enqueue_zrange(yas_session *s, cudaStream_t st) {
    prof_mark(s, kStZrange);
    launch_zrange(map_view(s->map), s->rc->cam, &s->fs->pp, s->zt, nullptr, st);
}

// Allocation, visibility and integration (Fuse, VoxelMap.cu:517-786), then the
// next frame's z-range tiles: beside integration on the side stream (they
// need only the visible list and the pose), after it when profiling.
// `dependent`: each of the three kernels is a programmatic dependent of the
// one before it (the frame step before allocation), except when profiling.
static void enqueue_fusion(yas_session *s, const int *skip, bool dependent) {
    MapDev v = map_view(s->map);
    const int fmt = s->map->cfg.voxel_format;
    cudaStream_t st = s->stream;
    dependent = dependent && !s->profiling;
    prof_mark(s, kStAllocate);
    launch_allocate(v, fmt, s->d_depth_m, s->cfg.width, s->cam, &s->fs->pp, skip, st, dependent);
    prof_mark(s, kStVisible);
    launch_visible(v, s->cam, &s->fs->pp, skip, st, dependent);
    const bool side = s->side && !s->profiling;
    if (side) {
        cudaEventRecord(s->ev_fork, st);
        cudaStreamWaitEvent(s->side, s->ev_fork, 0);
        enqueue_zrange(s, s->side);
    }
    prof_mark(s, kStIntegrate);
    launch_integrate(v, fmt, s->d_depth_m, s->cfg.width, s->cam, &s->fs->pp, skip, st, s->shape.integrate_ctas,
                     dependent);
    if (side) {
        cudaEventRecord(s->ev_join, s->side);
        cudaStreamWaitEvent(st, s->ev_join, 0);
    } else {
        enqueue_zrange(s, st);
    }
}

static void enqueue_first_frame(yas_session *s) {
    yas_tracker *tr = s->tr;
    tracker_image(tr, s->d_rgb, 3, s->cfg.width * 3, true, s->stream);
    tracker_depth(tr, s->d_depth, 1, s->cfg.width * 2, s->cfg.depth_scale, s->d_depth_m, true, s->stream);
    frame_begin_kernel<<<1, 32, 0, s->stream>>>(s->fs, pose_identity(), s->map->hdr);
    enqueue_fusion(s, nullptr, false);
    cudaMemcpyAsync(s->fs_host, s->fs, sizeof(FrameState), cudaMemcpyDeviceToHost, s->stream);
}

// Raycast of the map at the last pose and the model pyramid built from it
// (Tracking.cpp:164-169): reads the map, the pose pair and the z-range tiles
// the previous frame's fusion left, writes the reference set's vertex/normal
// maps only.
static void enqueue_raycast_branch(yas_session *s, cudaStream_t st) {
    yas_tracker *tr = s->tr;
    MapDev v = map_view(s->map);
    prof_mark(s, kStMarch);
    launch_march(v, s->map->cfg.voxel_format, s->rc->cam, &s->fs->pp, s->zt, tr->refb(0).vmap, s->cfg.width,
                 nullptr, st, s->shape.march_warps_x);
    prof_mark(s, kStModel);
    tracker_model(tr, st);
}

// Pyramids of the new frame (Tracking.cpp:172-173): read the frame, write the
// current set and the float depth only.
static void launch_input_copy(yas_session *s, cudaStream_t st);

static void enqueue_frame_branch(yas_session *s, cudaStream_t st) {
    yas_tracker *tr = s->tr;
    if (s->capture_input) launch_input_copy(s, st);
    prof_mark(s, kStImage);
    tracker_image(tr, s->d_rgb, 3, s->cfg.width * 3, false, st);
    prof_mark(s, kStDepth);
    tracker_depth(tr, s->d_depth, 1, s->cfg.width * 2, s->cfg.depth_scale, s->d_depth_m, false, st);
}

// A tracked frame up to the Gauss-Newton schedule: pyramids of the new frame,
// raycast of the map and model pyramid, GN state reset.
static void enqueue_pre(yas_session *s) {
    yas_tracker *tr = s->tr;
    cudaStream_t st = s->stream;
    if (s->side && !s->profiling) {
        // the two branches touch disjoint buffers: run them side by side; the
        // GN state reset (it reads neither branch's outputs) ends the shorter
        // frame branch, off the raycast's path
        cudaEventRecord(s->ev_fork, st);
        cudaStreamWaitEvent(s->side, s->ev_fork, 0);
        enqueue_raycast_branch(s, s->side);
        enqueue_frame_branch(s, st);
        launch_gn_init(tr, pose_identity(), st);
        cudaEventRecord(s->ev_join, s->side);
        cudaStreamWaitEvent(st, s->ev_join, 0);
    } else {
        enqueue_frame_branch(s, st);
        enqueue_raycast_branch(s, st);
        prof_mark(s, kStGnInit);
        launch_gn_init(tr, pose_identity(), st);
    }
}

// A tracked frame after the Gauss-Newton schedule: pose update (its result
// written to the host's copy too), fusion.  `dependent`: the fusion kernels
// are programmatic dependents (a lone session's frame; where sessions share
// the GPU, their waiting CTAs would hold slots other sessions' kernels need).
static void enqueue_post_as(yas_session *s, bool dependent) {
    cudaStream_t st = s->stream;
    prof_mark(s, kStFinalize);
    frame_finalize_kernel<<<1, 32, 0, st>>>(s->fs, s->tr->state, s->cfg.max_step_translation, s->map->hdr,
                                            s->fs_host_dev);
    enqueue_fusion(s, &s->fs->skip, dependent);
    prof_mark(s, kStEnd);
}

static void enqueue_post(yas_session *s) { enqueue_post_as(s, false); }

static void enqueue_tracked_frame(yas_session *s) {
    enqueue_pre(s);
    launch_gn_schedule(s->tr, s->stream);
    enqueue_post_as(s, true);
}

static int count_kernel_nodes(cudaGraph_t g, int *out) {
    size_t n = 0;
    YAS_TRY_CUDA(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    YAS_TRY_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
    int k = 0;
    for (size_t i = 0; i < n; ++i) {
        cudaGraphNodeType t;
        YAS_TRY_CUDA(cudaGraphNodeGetType(nodes[i], &t));
        if (t == cudaGraphNodeTypeKernel) ++k;
    }
    *out = k;
    return YAS_OK;
}

// Captures `fn` on the session stream into an executable graph; `kernels`
// (optional) receives its count of kernel nodes, `keep` (optional) the graph
// itself (destroyed otherwise).
static int capture_graph(yas_session *s, void (*fn)(yas_session *), cudaGraphExec_t *out, int *kernels,
                         cudaGraph_t *keep = nullptr) {
    cudaGraph_t g = nullptr;
    YAS_TRY_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    fn(s);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (e != cudaSuccess) {
        record_cuda_error(e, "graph capture", __FILE__, __LINE__);
        if (g) cudaGraphDestroy(g);
        return YAS_ERR_CUDA;
    }
    int st = kernels ? count_kernel_nodes(g, kernels) : YAS_OK;
    if (st == YAS_OK) {
        e = cudaGraphInstantiate(out, g, 0);
        if (e != cudaSuccess) {
            record_cuda_error(e, "graph instantiate", __FILE__, __LINE__);
            st = YAS_ERR_CUDA;
        }
    }
    if (st == YAS_OK && keep)
        *keep = g;
    else
        cudaGraphDestroy(g);
    return st;
}

// ---------------------------------------------------------------- frame input
static unsigned input_words(const yas_session *s) { return (unsigned)((size_t)s->cfg.width * s->cfg.height * 5 / 16); }

static cudaKernelNodeParams input_params(yas_session *s, const void **src, void **args, unsigned *n) {
    const size_t px = (size_t)s->cfg.width * s->cfg.height;
    n[0] = src[0] ? (unsigned)(px * 3 / 16) : 0u;
    n[1] = src[0] ? (unsigned)(px * 2 / 16) : 0u;
    args[0] = &src[0];
    args[1] = &src[1];
    args[2] = &s->d_rgb;
    args[3] = &s->d_depth;
    args[4] = &n[0];
    args[5] = &n[1];
    cudaKernelNodeParams p = {};
    p.func = (void *)input_copy_kernel;
    p.gridDim = dim3((input_words(s) + 255) / 256);
    p.blockDim = dim3(256);
    p.sharedMemBytes = 0;
    p.kernelParams = args;
    p.extra = nullptr;
    return p;
}

// The input copy node as captured: no sources (set before each launch).
static void launch_input_copy(yas_session *s, cudaStream_t st) {
    const uint4 *none = nullptr;
    input_copy_kernel<<<(input_words(s) + 255) / 256, 256, 0, st>>>(none, none, reinterpret_cast<uint4 *>(s->d_rgb),
                                                                   reinterpret_cast<uint4 *>(s->d_depth), 0u, 0u);
}

// Device address of `bytes` of a frame input the input copy kernel can read:
// 16-byte aligned memory of this device (on_device) or pinned host memory the
// device maps; null otherwise (the copy then runs on the stream).
static const void *readable_input(const yas_session *s, const void *p, size_t bytes, int on_device) {
    if ((reinterpret_cast<uintptr_t>(p) & 15u) || (bytes & 15u)) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    const bool ok = on_device ? (a.type == cudaMemoryTypeDevice && a.device == s->device)
                              : a.type == cudaMemoryTypeHost;
    return ok ? a.devicePointer : nullptr;
}

// Points the input copy node of exec[parity] at this frame's sources (null:
// the copies were enqueued on the stream and the node does nothing).
static int set_input_node(yas_session *s, int parity, const void *rgb, const void *depth) {
    if (s->input_src[parity][0] == rgb && s->input_src[parity][1] == depth) return YAS_OK;
    const void *src[2] = {rgb, depth};
    void *args[6];
    unsigned n[2];
    const cudaKernelNodeParams p = input_params(s, src, args, n);
    YAS_TRY_CUDA(cudaGraphExecKernelNodeSetParams(s->exec[parity], s->input_node[parity], &p));
    s->input_src[parity][0] = rgb;
    s->input_src[parity][1] = depth;
    return YAS_OK;
}

static int build_graph(yas_session *s, int parity) {
    s->capture_input = true;
    cudaGraph_t g = nullptr;
    const int st = capture_graph(s, enqueue_tracked_frame, &s->exec[parity], &s->kernels_per_frame, &g);
    s->capture_input = false;
    if (st != YAS_OK) return st;
    s->graph[parity] = g;
    s->input_node[parity] = nullptr;
    s->input_src[parity][0] = s->input_src[parity][1] = nullptr;
    size_t n = 0;
    YAS_TRY_CUDA(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    YAS_TRY_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
    for (size_t i = 0; i < n; ++i) {
        cudaGraphNodeType t;
        YAS_TRY_CUDA(cudaGraphNodeGetType(nodes[i], &t));
        if (t != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams p;
        YAS_TRY_CUDA(cudaGraphKernelNodeGetParams(nodes[i], &p));
        if (p.func == (void *)input_copy_kernel) s->input_node[parity] = nodes[i];
    }
    return YAS_OK;
}

// ---------------------------------------------------------------- interface for the request server
namespace yas {

int session_copy_input(yas_session *s, const uint8_t *rgb, const uint16_t *depth, int on_device) {
    const size_t n = (size_t)s->cfg.width * s->cfg.height;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    YAS_TRY_CUDA(cudaMemcpyAsync(s->d_rgb, rgb, n * 3, kind, s->stream));
    YAS_TRY_CUDA(cudaMemcpyAsync(s->d_depth, depth, n * 2, kind, s->stream));
    return YAS_OK;
}

bool session_needs_init(const yas_session *s) { return s->frames == 0; }

static void drop_graphs(yas_session *s) {
    for (int i = 0; i < 2; ++i) {
        if (s->exec[i]) cudaGraphExecDestroy(s->exec[i]);
        if (s->graph[i]) cudaGraphDestroy(s->graph[i]);
        if (s->pre_exec[i]) cudaGraphExecDestroy(s->pre_exec[i]);
        s->exec[i] = s->pre_exec[i] = nullptr;
        s->graph[i] = nullptr;
        s->input_node[i] = nullptr;
    }
    if (s->post_exec) cudaGraphExecDestroy(s->post_exec);
    s->post_exec = nullptr;
}

// Drops captured graphs that name map arrays which have since moved; a
// hibernated map cannot run frames.
static int check_graphs(yas_session *s) {
    if (s->map->hibernated) return YAS_ERR_STATE;
    const void *now[5] = {s->map->slots, s->map->block_keys, s->map->voxels, s->map->visible, s->map->hdr};
    bool same = true;
    for (int i = 0; i < 5; ++i) same = same && now[i] == s->graph_arrays[i];
    if (same) return YAS_OK;
    drop_graphs(s);
    for (int i = 0; i < 5; ++i) s->graph_arrays[i] = now[i];
    return YAS_OK;
}

int session_launch_first(yas_session *s) {
    YAS_TRY(check_graphs(s));
    enqueue_first_frame(s);
    YAS_TRY_CUDA(cudaGetLastError());
    s->frames++;
    return YAS_OK;
}

int session_launch_pre(yas_session *s) {
    YAS_TRY(check_graphs(s));
    const int parity = s->tr->cur;
    if (!s->pre_exec[parity]) YAS_TRY(capture_graph(s, enqueue_pre, &s->pre_exec[parity], nullptr));
    YAS_TRY_CUDA(cudaGraphLaunch(s->pre_exec[parity], s->stream));
    return YAS_OK;
}

int session_launch_post(yas_session *s) {
    YAS_TRY(check_graphs(s));
    if (!s->post_exec) YAS_TRY(capture_graph(s, enqueue_post, &s->post_exec, nullptr));
    YAS_TRY_CUDA(cudaGraphLaunch(s->post_exec, s->stream));
    s->tr->cur = 1 - s->tr->cur;
    s->frames++;
    return YAS_OK;
}

yas_tracker *session_tracker(yas_session *s) { return s->tr; }
cudaStream_t session_stream(yas_session *s) { return s->stream; }
yas_map *session_map_handle(yas_session *s) { return s->map; }
const yas_session_config &session_config(const yas_session *s) { return s->cfg; }

void session_set_shape(yas_session *s, const LaunchShape &shape) {
    s->shape = shape;
    drop_graphs(s);
}

const LaunchShape &session_shape(const yas_session *s) { return s->shape; }

void session_enqueue_first(yas_session *s) { enqueue_first_frame(s); }
void session_enqueue_pre(yas_session *s) { enqueue_pre(s); }
void session_enqueue_post(yas_session *s) { enqueue_post(s); }

void session_finish_first(yas_session *s) { s->frames++; }

void session_finish_tracked(yas_session *s) {
    s->tr->cur = 1 - s->tr->cur;
    s->frames++;
}

int session_restart(yas_session *s) {
    YAS_TRY_CUDA(cudaStreamSynchronize(s->stream));
    YAS_TRY(yas_map_reset(s->map));
    s->frames = 0;
    return YAS_OK;
}

void session_result(const yas_session *s, yas_pose *Tcm, int *status) {
    if (Tcm)
        for (int i = 0; i < 12; ++i) Tcm->m[i] = s->fs_host->Tcm[i];
    if (status) *status = s->fs_host->status;
}

}  // namespace yas

extern "C" {

YAS_API int yas_session_config_default(yas_session_config *cfg, int width, int height, const yas_intrinsics *K,
                                       int hash_slots, int max_blocks, float voxel_size, float trunc_dist,
                                       int voxel_format) {
    if (!cfg || !K) return YAS_ERR_BAD_ARG;
    memset(cfg, 0, sizeof(*cfg));
    cfg->width = width;
    cfg->height = height;
    cfg->K = *K;
    yas_map_config_default(&cfg->map, hash_slots, max_blocks, voxel_size, trunc_dist, voxel_format);
    cfg->num_levels = 3;
    const int it[5] = {10, 5, 3, 3, 3};
    for (int i = 0; i < 5; ++i) cfg->iterations[i] = it[i];
    cfg->mode = YAS_TRACK_RGBD;
    cfg->depth_scale = 0.001f;
    cfg->max_step_translation = 0.1f;
    cfg->use_graph = 1;
    cfg->fused_schedule = 1;
    return YAS_OK;
}

YAS_API int yas_session_destroy(yas_session *s);

YAS_API int yas_session_create(yas_session **out, const yas_session_config *cfg, void *stream) {
    if (!out || !cfg || cfg->width <= 0 || cfg->height <= 0) return YAS_ERR_BAD_ARG;
    *out = nullptr;
    yas_session *s = new yas_session();
    s->cfg = *cfg;
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return YAS_ERR_CUDA;
    }
    if (stream) {
        s->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            delete s;
            return YAS_ERR_CUDA;
        }
        s->own_stream = true;
    }
    s->cam = make_cam(cfg->K.fx, cfg->K.fy, cfg->K.cx, cfg->K.cy, cfg->width, cfg->height);
    int st = yas_map_create(&s->map, &cfg->map, &cfg->K, s->stream);
    if (st == YAS_OK) st = yas_raycaster_create(&s->rc, cfg->width, cfg->height, &cfg->K, s->stream);
    if (st == YAS_OK) {
        RaycastBuffers &z = s->zt;
        z.w = cfg->width;
        z.h = cfg->height;
        z.zw = (cfg->width + 7) / 8;
        z.zh = (cfg->height + 7) / 8;
        z.fw = (cfg->width + (1 << kFineShift) - 1) >> kFineShift;
        z.fh = (cfg->height + (1 << kFineShift) - 1) >> kFineShift;
        const size_t nz = (size_t)z.zw * z.zh;
        if (cudaMalloc(&z.znear, nz * 4) != cudaSuccess || cudaMalloc(&z.zfar, nz * 4) != cudaSuccess ||
            cudaMalloc(&z.queue, sizeof(unsigned)) != cudaSuccess ||
            cudaMalloc(&z.fnear, (size_t)z.fw * z.fh * 4) != cudaSuccess) {
            cudaGetLastError();
            st = YAS_ERR_OOM;
        }
    }
    if (st == YAS_OK) {
        const double K[9] = {cfg->K.fx, 0, cfg->K.cx, 0, cfg->K.fy, cfg->K.cy, 0, 0, 1};
        st = yas_tracker_create(&s->tr, cfg->width, cfg->height, K, cfg->num_levels, cfg->iterations, cfg->mode,
                                s->stream);
        if (st == YAS_OK) st = yas_tracker_set_schedule(s->tr, cfg->fused_schedule);
    }
    if (st == YAS_OK) {
        const size_t n = (size_t)cfg->width * cfg->height;
        if (cudaMalloc(&s->d_rgb, n * 3) != cudaSuccess || cudaMalloc(&s->d_depth, n * 2) != cudaSuccess ||
            cudaMalloc(&s->d_depth_m, n * 4) != cudaSuccess || cudaMalloc(&s->fs, sizeof(FrameState)) != cudaSuccess ||
            cudaMallocHost(&s->fs_host, sizeof(FrameState)) != cudaSuccess ||
            cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->fs_host_dev), s->fs_host, 0) != cudaSuccess) {
            cudaGetLastError();
            st = YAS_ERR_OOM;
        } else {
            cudaMemsetAsync(s->fs, 0, sizeof(FrameState), s->stream);
            memset(s->fs_host, 0, sizeof(FrameState));
        }
    }
    if (st == YAS_OK) {
        s->tr->hook = prof_mark;
        s->tr->hook_ctx = s;
        if (cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            st = YAS_ERR_CUDA;
        }
    }
    if (st == YAS_OK && cudaStreamSynchronize(s->stream) != cudaSuccess) st = YAS_ERR_CUDA;
    if (st != YAS_OK) {
        yas_session_destroy(s);
        return st;
    }
    *out = s;
    return YAS_OK;
}

YAS_API int yas_session_destroy(yas_session *s) {
    if (!s) return YAS_ERR_BAD_ARG;
    if (s->stream) cudaStreamSynchronize(s->stream);
    drop_graphs(s);
    if (s->tr) yas_tracker_destroy(s->tr);
    if (s->rc) yas_raycaster_destroy(s->rc);
    cudaFree(s->zt.znear);
    cudaFree(s->zt.zfar);
    cudaFree(s->zt.queue);
    cudaFree(s->zt.fnear);
    if (s->map) yas_map_destroy(s->map);
    cudaFree(s->d_rgb);
    cudaFree(s->d_depth);
    cudaFree(s->d_depth_m);
    cudaFree(s->fs);
    if (s->fs_host) cudaFreeHost(s->fs_host);
    if (s->side) {
        cudaStreamSynchronize(s->side);
        cudaStreamDestroy(s->side);
    }
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    if (s->own_stream) cudaStreamDestroy(s->stream);
    delete s;
    return YAS_OK;
}

YAS_API int yas_session_submit(yas_session *s, const uint8_t *rgb, const uint16_t *depth, int on_device) {
    if (!s || !rgb || !depth) return YAS_ERR_BAD_ARG;
    YAS_TRY(check_graphs(s));
    const size_t n = (size_t)s->cfg.width * s->cfg.height;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (s->frames > 0 && s->cfg.use_graph) {
        const int parity = s->tr->cur;
        if (!s->exec[parity]) YAS_TRY(build_graph(s, parity));
        // the graph's own input copy reads the sources where it can (off the
        // raycast's path); otherwise they are copied on the stream first
        const void *src_rgb = nullptr, *src_depth = nullptr;
        if (s->input_node[parity]) {
            src_rgb = readable_input(s, rgb, n * 3, on_device);
            src_depth = src_rgb ? readable_input(s, depth, n * 2, on_device) : nullptr;
            if (!src_depth) src_rgb = nullptr;
            YAS_TRY(set_input_node(s, parity, src_rgb, src_depth));
        }
        if (!src_rgb) {
            YAS_TRY_CUDA(cudaMemcpyAsync(s->d_rgb, rgb, n * 3, kind, s->stream));
            YAS_TRY_CUDA(cudaMemcpyAsync(s->d_depth, depth, n * 2, kind, s->stream));
        }
        YAS_TRY_CUDA(cudaGraphLaunch(s->exec[parity], s->stream));
        s->tr->cur = 1 - s->tr->cur;
        YAS_TRY_CUDA(cudaGetLastError());
        s->frames++;
        return YAS_OK;
    }
    YAS_TRY_CUDA(cudaMemcpyAsync(s->d_rgb, rgb, n * 3, kind, s->stream));
    YAS_TRY_CUDA(cudaMemcpyAsync(s->d_depth, depth, n * 2, kind, s->stream));
    if (s->frames == 0) {
        enqueue_first_frame(s);
    } else {
        enqueue_tracked_frame(s);
        s->tr->cur = 1 - s->tr->cur;
    }
    YAS_TRY_CUDA(cudaGetLastError());
    s->frames++;
    return YAS_OK;
}

YAS_API int yas_session_wait(yas_session *s, yas_pose *out_Tcm, int *out_status) {
    if (!s) return YAS_ERR_BAD_ARG;
    YAS_TRY_CUDA(cudaStreamSynchronize(s->stream));
    if (out_Tcm)
        for (int i = 0; i < 12; ++i) out_Tcm->m[i] = s->fs_host->Tcm[i];
    if (out_status) *out_status = s->fs_host->status;
    return YAS_OK;
}

YAS_API int yas_session_process_frame(yas_session *s, const uint8_t *rgb, const uint16_t *depth, int on_device,
                                      yas_pose *out_Tcm, int *out_status) {
    YAS_TRY(yas_session_submit(s, rgb, depth, on_device));
    return yas_session_wait(s, out_Tcm, out_status);
}

YAS_API int yas_session_map(yas_session *s, yas_map **out) {
    if (!s || !out) return YAS_ERR_BAD_ARG;
    *out = s->map;
    return YAS_OK;
}

YAS_API int yas_session_tracker(yas_session *s, yas_tracker **out) {
    if (!s || !out) return YAS_ERR_BAD_ARG;
    *out = s->tr;
    return YAS_OK;
}

YAS_API int yas_session_raycaster(yas_session *s, yas_raycaster **out) {
    if (!s || !out) return YAS_ERR_BAD_ARG;
    *out = s->rc;
    return YAS_OK;
}

YAS_API int yas_session_new_submap(yas_session *s, yas_map **out_previous) {
    if (!s || !out_previous) return YAS_ERR_BAD_ARG;
    YAS_TRY_CUDA(cudaStreamSynchronize(s->stream));
    if (s->side) YAS_TRY_CUDA(cudaStreamSynchronize(s->side));
    // camera pose in the world: T_world_map * Tcm of the last frame
    yas_pose Tw, Tcm;
    YAS_TRY(yas_map_get_pose(s->map, &Tw));
    for (int i = 0; i < 12; ++i) Tcm.m[i] = s->fs_host->Tcm[i];
    const Pose64 Tworld_cam = pose_mul(pose_from(Tw), pose_from(Tcm));
    yas_map *nm = nullptr;
    YAS_TRY(yas_map_create(&nm, &s->cfg.map, &s->cfg.K, s->stream));
    const yas_pose Tn = pose_to(Tworld_cam);
    yas_map_set_pose(nm, &Tn);
    yas_map_set_active(s->map, 0);
    *out_previous = s->map;
    s->map = nm;
    // captured frames name the previous map's arrays: capture again
    drop_graphs(s);
    // the frame's pose relative to the new submap restarts at the identity;
    // the next raycast's z-range tiles are the new (empty) map's
    frame_begin_kernel<<<1, 32, 0, s->stream>>>(s->fs, pose_identity(), nm->hdr);
    launch_zrange(map_view(nm), s->rc->cam, &s->fs->pp, s->zt, nullptr, s->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    YAS_TRY_CUDA(cudaMemcpyAsync(s->fs_host, s->fs, sizeof(FrameState), cudaMemcpyDeviceToHost, s->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(s->stream));
    return YAS_OK;
}

YAS_API int yas_session_frame_count(yas_session *s, int *out) {
    if (!s || !out) return YAS_ERR_BAD_ARG;
    *out = s->frames;
    return YAS_OK;
}

YAS_API int yas_session_depth(yas_session *s, const float **dev_depth, int *pitch_bytes) {
    if (!s || !dev_depth) return YAS_ERR_BAD_ARG;
    *dev_depth = s->d_depth_m;
    if (pitch_bytes) *pitch_bytes = s->cfg.width * 4;
    return YAS_OK;
}

YAS_API int yas_session_kernels_per_frame(yas_session *s, int *out) {
    if (!s || !out) return YAS_ERR_BAD_ARG;
    *out = s->kernels_per_frame;
    return YAS_OK;
}

YAS_API void *yas_session_stream(yas_session *s) { return s ? (void *)s->stream : nullptr; }

YAS_API int yas_session_profile_frame(yas_session *s, const uint8_t *rgb, const uint16_t *depth, int on_device,
                                      int *stage_ids, float *stage_ms, int capacity, int *out_count) {
    if (!s || !rgb || !depth || !out_count) return YAS_ERR_BAD_ARG;
    if (s->frames == 0) return YAS_ERR_STATE;  // the first frame initialises, it is not a tracked frame
    YAS_TRY(check_graphs(s));
    const size_t n = (size_t)s->cfg.width * s->cfg.height;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    YAS_TRY_CUDA(cudaMemcpyAsync(s->d_rgb, rgb, n * 3, kind, s->stream));
    YAS_TRY_CUDA(cudaMemcpyAsync(s->d_depth, depth, n * 2, kind, s->stream));
    s->profiling = true;
    enqueue_tracked_frame(s);
    s->profiling = false;
    s->tr->cur = 1 - s->tr->cur;
    s->frames++;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    int st = YAS_OK;
    if (e != cudaSuccess) {
        record_cuda_error(e, "profile frame", __FILE__, __LINE__);
        st = YAS_ERR_CUDA;
    }
    const int m = (int)s->prof_events.size() - 1;
    int k = 0;
    for (int i = 0; i < m && st == YAS_OK; ++i) {
        if (k >= capacity) {
            st = YAS_ERR_CAPACITY;
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, s->prof_events[i], s->prof_events[i + 1]);
        if (stage_ids) stage_ids[k] = s->prof_ids[i];
        if (stage_ms) stage_ms[k] = ms;
        ++k;
    }
    for (cudaEvent_t ev : s->prof_events) cudaEventDestroy(ev);
    s->prof_events.clear();
    s->prof_ids.clear();
    *out_count = k;
    return st;
}

}  // extern "C"
