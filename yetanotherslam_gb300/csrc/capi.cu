// capi.cu — extern "C" entry points of libyas_gb300 for the map, raycaster,
// mesher and tracker handles (declared in include/yas.h), and the host pose
// algebra shared by the library.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "yas_track.h"

namespace yas {

static thread_local char g_last_error[512];

void record_cuda_error(cudaError_t e, const char *expr, const char *file, int line) {
    snprintf(g_last_error, sizeof(g_last_error), "%s at %s:%d: %s", cudaGetErrorString(e), file, line, expr);
}

Pose64 pose_identity() {
    Pose64 p;
    for (int i = 0; i < 9; ++i) p.r[i] = (i % 4 == 0) ? 1.0 : 0.0;
    p.t[0] = p.t[1] = p.t[2] = 0.0;
    return p;
}

Pose64 pose_from(const yas_pose &q) {
    Pose64 p;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) p.r[i * 3 + j] = q.m[i * 4 + j];
        p.t[i] = q.m[i * 4 + 3];
    }
    return p;
}

yas_pose pose_to(const Pose64 &p) {
    yas_pose q;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) q.m[i * 4 + j] = p.r[i * 3 + j];
        q.m[i * 4 + 3] = p.t[i];
    }
    return q;
}

Pose64 pose_inverse(const Pose64 &p) {
    Pose64 o;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) o.r[i * 3 + j] = p.r[j * 3 + i];
    for (int i = 0; i < 3; ++i) o.t[i] = -((p.r[0 * 3 + i] * p.t[0] + p.r[1 * 3 + i] * p.t[1]) + p.r[2 * 3 + i] * p.t[2]);
    return o;
}

Pose64 pose_mul(const Pose64 &a, const Pose64 &b) {
    Pose64 o;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            o.r[i * 3 + j] = (a.r[i * 3 + 0] * b.r[0 * 3 + j] + a.r[i * 3 + 1] * b.r[1 * 3 + j]) + a.r[i * 3 + 2] * b.r[2 * 3 + j];
        o.t[i] = ((a.r[i * 3 + 0] * b.t[0] + a.r[i * 3 + 1] * b.t[1]) + a.r[i * 3 + 2] * b.t[2]) + a.t[i];
    }
    return o;
}

Rigid32 rigid_from(const Pose64 &p) {
    Rigid32 r;
    for (int i = 0; i < 9; ++i) r.r[i] = (float)p.r[i];
    for (int i = 0; i < 3; ++i) r.t[i] = (float)p.t[i];
    return r;
}

Cam make_cam(float fx, float fy, float cx, float cy, int w, int h) {
    Cam c;
    c.fx = fx;
    c.fy = fy;
    c.cx = cx;
    c.cy = cy;
    c.invfx = (float)(1.0 / (double)fx);
    c.invfy = (float)(1.0 / (double)fy);
    c.w = w;
    c.h = h;
    return c;
}

static PosePair make_pair(const yas_pose *Tcm) {
    Pose64 p = pose_from(*Tcm);
    PosePair pp;
    pp.T = rigid_from(p);
    pp.Tinv = rigid_from(pose_inverse(p));
    return pp;
}

static bool is_pow2(long long v) { return v > 0 && (v & (v - 1)) == 0; }

// Device staging buffer for host inputs, grown on demand.
struct Staging {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t n) {
        if (n <= bytes) return YAS_OK;
        cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        if (cudaMalloc(&ptr, n) != cudaSuccess) {
            cudaGetLastError();
            return YAS_ERR_OOM;
        }
        bytes = n;
        return YAS_OK;
    }
    ~Staging() { cudaFree(ptr); }
};

}  // namespace yas

using namespace yas;

// Per-map staging for host depth in yas_map_fuse_depth.
struct MapExtra {
    Staging depth;
};
static std::mutex g_extra_mutex;
#include <unordered_map>
static std::unordered_map<const yas_map *, MapExtra *> g_map_extra;
static MapExtra *map_extra(const yas_map *m) {
    std::lock_guard<std::mutex> lk(g_extra_mutex);
    auto it = g_map_extra.find(m);
    if (it != g_map_extra.end()) return it->second;
    MapExtra *e = new MapExtra();
    g_map_extra[m] = e;
    return e;
}
static void map_extra_drop(const yas_map *m) {
    std::lock_guard<std::mutex> lk(g_extra_mutex);
    auto it = g_map_extra.find(m);
    if (it != g_map_extra.end()) {
        delete it->second;
        g_map_extra.erase(it);
    }
}

extern "C" {

YAS_API const char *yas_status_string(int s) {
    switch (s) {
        case YAS_OK: return "ok";
        case YAS_ERR_BAD_ARG: return "bad argument";
        case YAS_ERR_OOM: return "out of memory";
        case YAS_ERR_CUDA: return g_last_error[0] ? g_last_error : "cuda error";
        case YAS_ERR_TABLE_FULL: return "hash table probe limit reached";
        case YAS_ERR_POOL_FULL: return "voxel block pool exhausted";
        case YAS_ERR_NUMERIC: return "NaN in Gauss-Newton solve";
        case YAS_ERR_TRACK_LOST: return "frame step above the translation limit";
        case YAS_ERR_MESH_OVERFLOW: return "triangle buffer overflow";
        case YAS_ERR_STATE: return "invalid state for this call";
        case YAS_ERR_COORD_RANGE: return "block coordinate outside the key range";
        case YAS_ERR_CAPACITY: return "caller buffer too small";
        case YAS_ERR_TIMEOUT: return "device-side wait timed out";
        case YAS_ERR_IO: return "file could not be read or written";
        default: return "unknown status";
    }
}

YAS_API const char *yas_version(void) { return "yas-gb300 0.1.0 sm_103a"; }

// ------------------------------------------------------------------ map
YAS_API int yas_map_config_default(yas_map_config *cfg, int hash_slots, int max_blocks, float voxel_size,
                                   float trunc_dist, int voxel_format) {
    if (!cfg) return YAS_ERR_BAD_ARG;
    cfg->hash_slots = hash_slots;
    cfg->max_blocks = max_blocks;
    cfg->voxel_size = voxel_size;
    cfg->trunc_dist = trunc_dist;
    cfg->depth_min = 0.1f;
    cfg->depth_max = 3.0f;
    cfg->voxel_format = voxel_format;
    cfg->max_weight = 255;
    return YAS_OK;
}

YAS_API int yas_map_create(yas_map **out, const yas_map_config *cfg, const yas_intrinsics *K, void *stream) {
    if (!out || !cfg || !K) return YAS_ERR_BAD_ARG;
    *out = nullptr;
    if (!is_pow2(cfg->hash_slots) || cfg->max_blocks <= 0 || !(cfg->voxel_size > 0.0f) ||
        !(cfg->trunc_dist > 0.0f) || cfg->voxel_format < 0 || cfg->voxel_format > 3 || cfg->max_weight < 1 ||
        cfg->max_weight > 65535 || (cfg->voxel_format != YAS_VOXEL_F32 && cfg->max_weight > 255))
        return YAS_ERR_BAD_ARG;
    yas_map *m = new yas_map();
    m->cfg = *cfg;
    m->cam_K = make_cam(K->fx, K->fy, K->cx, K->cy, 0, 0);
    m->stream = (cudaStream_t)stream;
    m->Tcw = pose_identity();
    int st = map_dev_alloc(m);
    if (st != YAS_OK) {
        delete m;
        return st;
    }
    if (cudaMalloc(&m->pose_dev, sizeof(PosePair)) != cudaSuccess ||
        cudaMallocHost(&m->hdr_host, sizeof(MapHeader)) != cudaSuccess) {
        cudaGetLastError();
        map_dev_free(m);
        cudaFree(m->pose_dev);
        delete m;
        return YAS_ERR_OOM;
    }
    launch_map_reset(map_view(m), m->stream);
    cudaError_t e = cudaStreamSynchronize(m->stream);
    if (e != cudaSuccess) {
        record_cuda_error(e, "reset", __FILE__, __LINE__);
        yas_map_destroy(m);
        return YAS_ERR_CUDA;
    }
    *out = m;
    return YAS_OK;
}

YAS_API int yas_map_create_ref(yas_map **out, int hashTableSize, int bucketSize, int voxelBlockSize,
                               float voxelSize, float truncationDist, const yas_intrinsics *K, void *stream) {
    if (hashTableSize <= 0 || bucketSize <= 0 || voxelBlockSize <= 0) return YAS_ERR_BAD_ARG;
    long long want = hashTableSize > 2LL * voxelBlockSize ? hashTableSize : 2LL * voxelBlockSize;
    long long slots = 1;
    while (slots < want) slots <<= 1;
    if (slots > (1LL << 30)) return YAS_ERR_BAD_ARG;
    yas_map_config cfg;
    yas_map_config_default(&cfg, (int)slots, voxelBlockSize, voxelSize, truncationDist, YAS_VOXEL_F32);
    return yas_map_create(out, &cfg, K, stream);
}

YAS_API int yas_map_destroy(yas_map *m) {
    if (!m) return YAS_ERR_BAD_ARG;
    cudaStreamSynchronize(m->stream);
    map_dev_free(m);
    cudaFree(m->pose_dev);
    if (m->hdr_host) cudaFreeHost(m->hdr_host);
    map_extra_drop(m);
    delete m;
    return YAS_OK;
}

YAS_API int yas_map_reset(yas_map *m) {
    if (!m) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    launch_map_reset(map_view(m), m->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}

static int read_header(yas_map *m) {
    YAS_TRY_CUDA(cudaMemcpyAsync(m->hdr_host, m->hdr, sizeof(MapHeader), cudaMemcpyDeviceToHost, m->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));
    return YAS_OK;
}

YAS_API int yas_map_empty(yas_map *m, int *out) {
    if (!m || !out) return YAS_ERR_BAD_ARG;
    if (m->hibernated) {
        *out = m->hib_hdr.n_alloc == 0;
        return YAS_OK;
    }
    YAS_TRY(read_header(m));
    *out = m->hdr_host->n_alloc == 0;
    return YAS_OK;
}

YAS_API int yas_map_fuse_depth(yas_map *m, const float *depth, int width, int height, int pitch_bytes,
                               int on_device, const yas_pose *Tcm) {
    if (!m || !depth || !Tcm || width <= 0 || height <= 0 || pitch_bytes < width * 4 || (pitch_bytes & 3))
        return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    const float *d = depth;
    if (!on_device) {
        MapExtra *ex = map_extra(m);
        YAS_TRY(ex->depth.ensure((size_t)pitch_bytes * height));
        YAS_TRY_CUDA(cudaMemcpyAsync(ex->depth.ptr, depth, (size_t)pitch_bytes * height, cudaMemcpyHostToDevice,
                                     m->stream));
        d = (const float *)ex->depth.ptr;
    }
    PosePair pp = make_pair(Tcm);
    YAS_TRY_CUDA(cudaMemcpyAsync(m->pose_dev, &pp, sizeof(pp), cudaMemcpyHostToDevice, m->stream));
    Cam cam = make_cam(m->cam_K.fx, m->cam_K.fy, m->cam_K.cx, m->cam_K.cy, width, height);
    MapDev v = map_view(m);
    launch_allocate(v, m->cfg.voxel_format, d, pitch_bytes / 4, cam, m->pose_dev, nullptr, m->stream);
    YAS_TRY_CUDA(cudaMemsetAsync(&m->hdr->n_visible, 0, sizeof(unsigned), m->stream));
    launch_visible(v, cam, m->pose_dev, nullptr, m->stream);
    launch_integrate(v, m->cfg.voxel_format, d, pitch_bytes / 4, cam, m->pose_dev, nullptr, m->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    if (!on_device) YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));  // staging reuse safety
    return YAS_OK;
}

YAS_API int yas_map_check_visible(yas_map *m, int cols, int rows, const yas_pose *Tcm, unsigned *out) {
    if (!m || !Tcm || cols <= 0 || rows <= 0) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    PosePair pp = make_pair(Tcm);
    YAS_TRY_CUDA(cudaMemcpyAsync(m->pose_dev, &pp, sizeof(pp), cudaMemcpyHostToDevice, m->stream));
    YAS_TRY_CUDA(cudaMemsetAsync(&m->hdr->n_visible, 0, sizeof(unsigned), m->stream));
    Cam cam = make_cam(m->cam_K.fx, m->cam_K.fy, m->cam_K.cx, m->cam_K.cy, cols, rows);
    launch_visible(map_view(m), cam, m->pose_dev, nullptr, m->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    if (out) {
        YAS_TRY(read_header(m));
        *out = m->hdr_host->n_visible;
    }
    return YAS_OK;
}

YAS_API int yas_map_num_visible(yas_map *m, unsigned *out) {
    if (!m || !out) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    YAS_TRY(read_header(m));
    *out = m->hdr_host->n_visible;
    return YAS_OK;
}

YAS_API int yas_map_reset_visible(yas_map *m) {
    if (!m) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    YAS_TRY_CUDA(cudaMemsetAsync(&m->hdr->n_visible, 0, sizeof(unsigned), m->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));
    return YAS_OK;
}

YAS_API int yas_map_num_allocated(yas_map *m, unsigned *out) {
    if (!m || !out) return YAS_ERR_BAD_ARG;
    if (m->hibernated) {
        *out = m->hib_hdr.n_alloc < (unsigned)m->cfg.max_blocks ? m->hib_hdr.n_alloc : (unsigned)m->cfg.max_blocks;
        return YAS_OK;
    }
    YAS_TRY(read_header(m));
    unsigned n = m->hdr_host->n_alloc;
    *out = n < (unsigned)m->cfg.max_blocks ? n : (unsigned)m->cfg.max_blocks;
    return YAS_OK;
}

YAS_API int yas_map_take_errors(yas_map *m, unsigned *out_bits) {
    if (!m || !out_bits) return YAS_ERR_BAD_ARG;
    if (m->hibernated) {
        *out_bits = 0;
        return YAS_OK;
    }
    YAS_TRY(read_header(m));
    *out_bits = m->hdr_host->err_bits;
    YAS_TRY_CUDA(cudaMemsetAsync(&m->hdr->err_bits, 0, sizeof(unsigned), m->stream));
    return YAS_OK;
}

YAS_API int yas_map_export(yas_map *m, int *coords, float *sdf, float *weight, unsigned capacity,
                           unsigned *out_count) {
    if (!m || !out_count) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    unsigned n;
    YAS_TRY(yas_map_num_allocated(m, &n));
    *out_count = n;
    if (!coords || !sdf || !weight) return YAS_OK;  // size query
    if (capacity < n) return YAS_ERR_CAPACITY;
    const unsigned chunk = 8192;
    int *dc = nullptr;
    float *ds = nullptr, *dw = nullptr;
    if (cudaMalloc(&dc, (size_t)chunk * 12) != cudaSuccess || cudaMalloc(&ds, (size_t)chunk * 512 * 4) != cudaSuccess ||
        cudaMalloc(&dw, (size_t)chunk * 512 * 4) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(dc);
        cudaFree(ds);
        cudaFree(dw);
        return YAS_ERR_OOM;
    }
    int st = YAS_OK;
    for (unsigned first = 0; first < n && st == YAS_OK; first += chunk) {
        unsigned cnt = n - first < chunk ? n - first : chunk;
        launch_map_export(map_view(m), m->cfg.voxel_format, dc, ds, dw, first, cnt, m->stream);
        if (cudaMemcpyAsync(coords + (size_t)first * 3, dc, (size_t)cnt * 12, cudaMemcpyDeviceToHost, m->stream) !=
                cudaSuccess ||
            cudaMemcpyAsync(sdf + (size_t)first * 512, ds, (size_t)cnt * 2048, cudaMemcpyDeviceToHost, m->stream) !=
                cudaSuccess ||
            cudaMemcpyAsync(weight + (size_t)first * 512, dw, (size_t)cnt * 2048, cudaMemcpyDeviceToHost,
                            m->stream) != cudaSuccess ||
            cudaStreamSynchronize(m->stream) != cudaSuccess) {
            record_cuda_error(cudaGetLastError(), "export", __FILE__, __LINE__);
            st = YAS_ERR_CUDA;
        }
    }
    cudaFree(dc);
    cudaFree(ds);
    cudaFree(dw);
    return st;
}

YAS_API int yas_map_import(yas_map *m, const int *coords, const float *sdf, const float *weight, unsigned count) {
    if (!m || (count && (!coords || !sdf || !weight))) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    if (count == 0) return YAS_OK;
    int *dc = nullptr;
    float *ds = nullptr, *dw = nullptr;
    if (cudaMalloc(&dc, (size_t)count * 12) != cudaSuccess || cudaMalloc(&ds, (size_t)count * 2048) != cudaSuccess ||
        cudaMalloc(&dw, (size_t)count * 2048) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(dc);
        cudaFree(ds);
        cudaFree(dw);
        return YAS_ERR_OOM;
    }
    int st = YAS_OK;
    if (cudaMemcpyAsync(dc, coords, (size_t)count * 12, cudaMemcpyHostToDevice, m->stream) != cudaSuccess ||
        cudaMemcpyAsync(ds, sdf, (size_t)count * 2048, cudaMemcpyHostToDevice, m->stream) != cudaSuccess ||
        cudaMemcpyAsync(dw, weight, (size_t)count * 2048, cudaMemcpyHostToDevice, m->stream) != cudaSuccess) {
        st = YAS_ERR_CUDA;
    } else {
        launch_map_import(map_view(m), m->cfg.voxel_format, dc, ds, dw, count, m->stream);
        if (cudaStreamSynchronize(m->stream) != cudaSuccess) st = YAS_ERR_CUDA;
    }
    if (st != YAS_OK) record_cuda_error(cudaGetLastError(), "import", __FILE__, __LINE__);
    cudaFree(dc);
    cudaFree(ds);
    cudaFree(dw);
    return st;
}

YAS_API int yas_map_export_visible(yas_map *m, int *coords, unsigned capacity, unsigned *out_count) {
    if (!m || !out_count) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    YAS_TRY(read_header(m));
    unsigned n = m->hdr_host->n_visible;
    *out_count = n;
    if (!coords) return YAS_OK;
    if (capacity < n) return YAS_ERR_CAPACITY;
    if (n == 0) return YAS_OK;
    int *dc = nullptr;
    if (cudaMalloc(&dc, (size_t)n * 12) != cudaSuccess) {
        cudaGetLastError();
        return YAS_ERR_OOM;
    }
    launch_visible_coords(map_view(m), dc, n, m->stream);
    cudaError_t e = cudaMemcpyAsync(coords, dc, (size_t)n * 12, cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    cudaFree(dc);
    if (e != cudaSuccess) {
        record_cuda_error(e, "export_visible", __FILE__, __LINE__);
        return YAS_ERR_CUDA;
    }
    return YAS_OK;
}

YAS_API int yas_map_get_pose(yas_map *m, yas_pose *out) {
    if (!m || !out) return YAS_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(m->pose_mutex);
    *out = pose_to(m->Tcw);
    return YAS_OK;
}

YAS_API int yas_map_set_pose(yas_map *m, const yas_pose *T) {
    if (!m || !T) return YAS_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(m->pose_mutex);
    m->Tcw = pose_from(*T);
    return YAS_OK;
}

YAS_API int yas_map_set_active(yas_map *m, int flag) {
    if (!m) return YAS_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(m->active_mutex);
    m->active = flag != 0;
    return YAS_OK;
}

YAS_API int yas_map_is_active(yas_map *m, int *out) {
    if (!m || !out) return YAS_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(m->active_mutex);
    *out = m->active ? 1 : 0;
    return YAS_OK;
}

YAS_API int yas_map_hibernate(yas_map *m) {
    if (!m) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_OK;
    YAS_TRY(read_header(m));
    m->hib_hdr = *m->hdr_host;
    const size_t nslots = (size_t)m->cfg.hash_slots;
    unsigned n = m->hib_hdr.n_alloc < (unsigned)m->cfg.max_blocks ? m->hib_hdr.n_alloc : (unsigned)m->cfg.max_blocks;
    const size_t vb = (size_t)kBlockVoxels * (m->cfg.voxel_format == YAS_VOXEL_F32 ? 8 : 4);
    m->hib_slots.resize(nslots * sizeof(HashSlot));
    m->hib_keys.resize((size_t)n * 8);
    m->hib_voxels.resize((size_t)n * vb);
    // the visible list of the last fusion (the next raycast starts from it)
    const unsigned nv = std::min(m->hib_hdr.n_visible, (unsigned)m->cfg.max_blocks);
    m->hib_visible.resize((size_t)nv * sizeof(int));
    YAS_TRY_CUDA(cudaMemcpyAsync(m->hib_slots.data(), m->slots, m->hib_slots.size(), cudaMemcpyDeviceToHost, m->stream));
    if (nv)
        YAS_TRY_CUDA(cudaMemcpyAsync(m->hib_visible.data(), m->visible, m->hib_visible.size(), cudaMemcpyDeviceToHost,
                                     m->stream));
    if (n) {
        YAS_TRY_CUDA(cudaMemcpyAsync(m->hib_keys.data(), m->block_keys, m->hib_keys.size(), cudaMemcpyDeviceToHost,
                                     m->stream));
        YAS_TRY_CUDA(cudaMemcpyAsync(m->hib_voxels.data(), m->voxels, m->hib_voxels.size(), cudaMemcpyDeviceToHost,
                                     m->stream));
    }
    YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));
    map_dev_free(m);
    m->hibernated = true;
    return YAS_OK;
}

YAS_API int yas_map_reactivate(yas_map *m) {
    if (!m) return YAS_ERR_BAD_ARG;
    if (!m->hibernated) return YAS_OK;
    YAS_TRY(map_dev_alloc(m));
    YAS_TRY_CUDA(cudaMemcpyAsync(m->slots, m->hib_slots.data(), m->hib_slots.size(), cudaMemcpyHostToDevice, m->stream));
    if (!m->hib_keys.empty()) {
        YAS_TRY_CUDA(cudaMemcpyAsync(m->block_keys, m->hib_keys.data(), m->hib_keys.size(), cudaMemcpyHostToDevice,
                                     m->stream));
        YAS_TRY_CUDA(cudaMemcpyAsync(m->voxels, m->hib_voxels.data(), m->hib_voxels.size(), cudaMemcpyHostToDevice,
                                     m->stream));
    }
    MapHeader h = m->hib_hdr;
    h.n_visible = (unsigned)(m->hib_visible.size() / sizeof(int));
    if (h.n_visible)
        YAS_TRY_CUDA(cudaMemcpyAsync(m->visible, m->hib_visible.data(), m->hib_visible.size(), cudaMemcpyHostToDevice,
                                     m->stream));
    YAS_TRY_CUDA(cudaMemcpyAsync(m->hdr, &h, sizeof(h), cudaMemcpyHostToDevice, m->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));
    m->hib_visible.clear();
    m->hib_visible.shrink_to_fit();
    m->hib_slots.clear();
    m->hib_slots.shrink_to_fit();
    m->hib_keys.clear();
    m->hib_keys.shrink_to_fit();
    m->hib_voxels.clear();
    m->hib_voxels.shrink_to_fit();
    m->hibernated = false;
    return YAS_OK;
}

YAS_API int yas_map_is_hibernated(yas_map *m, int *out) {
    if (!m || !out) return YAS_ERR_BAD_ARG;
    *out = m->hibernated ? 1 : 0;
    return YAS_OK;
}

YAS_API int yas_map_device_bytes(yas_map *m, size_t *out) {
    if (!m || !out) return YAS_ERR_BAD_ARG;
    *out = m->hibernated ? 0
                         : (size_t)m->cfg.hash_slots * sizeof(HashSlot) + (size_t)m->cfg.max_blocks * (8 + 4) +
                               m->voxel_bytes() + sizeof(MapHeader) + sizeof(PosePair);
    return YAS_OK;
}

// ------------------------------------------------------------------ submap file
static int map_grow(yas_map *m, long long want_slots, long long want_blocks);

// Binary submap file (little-endian): SubmapFileHeader, then n_blocks block
// coordinates (int32 x, y, z), then n_blocks * 512 voxels in the map's own
// storage format (8 bytes for F32, 4 for F16 and S24), pool order.
struct SubmapFileHeader {
    char magic[8];          // "YASSUBM1"
    uint32_t version;       // 3 (F16 voxels: half + FP32-bit residual + u8 weight)
    uint32_t voxel_format;  // enum yas_voxel_format
    float voxel_size, trunc_dist, depth_min, depth_max;
    int32_t max_weight, hash_slots, max_blocks;
    uint32_t n_blocks;
    double pose[12];        // map pose (Tcw), row-major [R | t]
};
static_assert(sizeof(SubmapFileHeader) == 144, "submap file header layout");
static const char kSubmapMagic[8] = {'Y', 'A', 'S', 'S', 'U', 'B', 'M', '1'};

extern "C" {

YAS_API int yas_map_save(yas_map *m, const char *path) {
    if (!m || !path) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    YAS_TRY(read_header(m));
    const unsigned n = std::min(m->hdr_host->n_alloc, (unsigned)m->cfg.max_blocks);
    const size_t vb = (size_t)kBlockVoxels * (m->cfg.voxel_format == YAS_VOXEL_F32 ? 8 : 4);
    std::vector<unsigned long long> keys(n);
    std::vector<unsigned char> vox((size_t)n * vb);
    if (n) {
        YAS_TRY_CUDA(cudaMemcpyAsync(keys.data(), m->block_keys, (size_t)n * 8, cudaMemcpyDeviceToHost, m->stream));
        YAS_TRY_CUDA(cudaMemcpyAsync(vox.data(), m->voxels, vox.size(), cudaMemcpyDeviceToHost, m->stream));
        YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));
    }
    SubmapFileHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kSubmapMagic, 8);
    h.version = 3;
    h.voxel_format = (uint32_t)m->cfg.voxel_format;
    h.voxel_size = m->cfg.voxel_size;
    h.trunc_dist = m->cfg.trunc_dist;
    h.depth_min = m->cfg.depth_min;
    h.depth_max = m->cfg.depth_max;
    h.max_weight = m->cfg.max_weight;
    h.hash_slots = m->cfg.hash_slots;
    h.max_blocks = m->cfg.max_blocks;
    h.n_blocks = n;
    {
        std::lock_guard<std::mutex> lk(m->pose_mutex);
        const yas_pose p = pose_to(m->Tcw);
        memcpy(h.pose, p.m, sizeof(h.pose));
    }
    std::vector<int32_t> coords((size_t)n * 3);
    for (unsigned i = 0; i < n; ++i) unpack_key(keys[i], coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]);
    FILE *f = fopen(path, "wb");
    if (!f) return YAS_ERR_IO;
    bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
    if (ok && n) ok = fwrite(coords.data(), sizeof(int32_t), coords.size(), f) == coords.size();
    if (ok && n) ok = fwrite(vox.data(), 1, vox.size(), f) == vox.size();
    ok = (fclose(f) == 0) && ok;
    return ok ? YAS_OK : YAS_ERR_IO;
}

YAS_API int yas_map_load(yas_map *m, const char *path) {
    if (!m || !path) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    FILE *f = fopen(path, "rb");
    if (!f) return YAS_ERR_IO;
    SubmapFileHeader h;
    bool ok = fread(&h, sizeof(h), 1, f) == 1 && memcmp(h.magic, kSubmapMagic, 8) == 0 && h.version == 3;
    const size_t vb = (size_t)kBlockVoxels * (h.voxel_format == YAS_VOXEL_F32 ? 8 : 4);
    std::vector<int32_t> coords;
    std::vector<unsigned char> vox;
    if (ok) {
        // the block count is checked against the file's length before it sizes anything
        const long here = ftell(f);
        ok = here >= 0 && fseek(f, 0, SEEK_END) == 0;
        const long end = ok ? ftell(f) : -1;
        ok = ok && end >= here && fseek(f, here, SEEK_SET) == 0 && h.n_blocks <= (1u << 30) &&
             (unsigned long long)(end - here) == (unsigned long long)h.n_blocks * (12ull + vb);
    }
    if (ok) {
        coords.resize((size_t)h.n_blocks * 3);
        vox.resize((size_t)h.n_blocks * vb);
        if (h.n_blocks)
            ok = fread(coords.data(), sizeof(int32_t), coords.size(), f) == coords.size() &&
                 fread(vox.data(), 1, vox.size(), f) == vox.size();
    }
    fclose(f);
    if (!ok) return YAS_ERR_IO;
    if ((int)h.voxel_format != m->cfg.voxel_format || h.voxel_size != m->cfg.voxel_size) return YAS_ERR_BAD_ARG;
    const unsigned n = h.n_blocks;
    std::vector<unsigned long long> keys(n);
    for (unsigned i = 0; i < n; ++i) {
        if (!coord_in_range(coords[3 * i], coords[3 * i + 1], coords[3 * i + 2])) return YAS_ERR_COORD_RANGE;
        keys[i] = pack_key(coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]);
    }
    YAS_TRY(yas_map_reset(m));
    YAS_TRY(map_grow(m, std::max<long long>(h.hash_slots, 2LL * n), std::max<long long>(h.max_blocks, n)));
    if (n) {
        YAS_TRY_CUDA(cudaMemcpyAsync(m->block_keys, keys.data(), (size_t)n * 8, cudaMemcpyHostToDevice, m->stream));
        YAS_TRY_CUDA(cudaMemcpyAsync(m->voxels, vox.data(), vox.size(), cudaMemcpyHostToDevice, m->stream));
        YAS_TRY_CUDA(cudaMemcpyAsync(&m->hdr->n_alloc, &n, sizeof(unsigned), cudaMemcpyHostToDevice, m->stream));
        launch_rehash(map_view(m), n, m->stream);
        YAS_TRY_CUDA(cudaGetLastError());
    }
    YAS_TRY(read_header(m));
    if (m->hdr_host->err_bits & err_bit(YAS_ERR_TABLE_FULL)) return YAS_ERR_TABLE_FULL;
    yas_pose p;
    memcpy(p.m, h.pose, sizeof(p.m));
    std::lock_guard<std::mutex> lk(m->pose_mutex);
    m->Tcw = pose_from(p);
    return YAS_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ shading
extern "C" {

YAS_API int yas_copy_to_host(void *dst, int dpitch, const void *src, int spitch, int width_bytes, int height) {
    if (!dst || !src || width_bytes <= 0 || height <= 0 || dpitch < width_bytes || spitch < width_bytes)
        return YAS_ERR_BAD_ARG;
    YAS_TRY_CUDA(cudaMemcpy2D(dst, (size_t)dpitch, src, (size_t)spitch, (size_t)width_bytes, (size_t)height,
                              cudaMemcpyDefault));
    return YAS_OK;
}

YAS_API int yas_render_scene(const float *dev_vmap, const float *dev_nmap, int width, int height, int pitch_bytes,
                             const float *light, uint8_t *rgba, int out_pitch_bytes, int on_device, void *stream) {
    if (!dev_vmap || !dev_nmap || !rgba || width <= 0 || height <= 0 || pitch_bytes < width * 16 ||
        (pitch_bytes & 15) || out_pitch_bytes < width * 4 || (out_pitch_bytes & 3))
        return YAS_ERR_BAD_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const float3 L = light ? make_float3(light[0], light[1], light[2]) : make_float3(5.0f, 5.0f, 5.0f);
    uchar4 *out = reinterpret_cast<uchar4 *>(rgba);
    void *tmp = nullptr;
    if (!on_device) {
        YAS_TRY_CUDA(cudaMallocAsync(&tmp, (size_t)out_pitch_bytes * height, s));
        out = static_cast<uchar4 *>(tmp);
    }
    launch_render_scene(reinterpret_cast<const float4 *>(dev_vmap), reinterpret_cast<const float4 *>(dev_nmap),
                        pitch_bytes / 16, width, height, L, out, out_pitch_bytes / 4, s);
    cudaError_t e = cudaGetLastError();
    if (!on_device) {
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(rgba, tmp, (size_t)out_pitch_bytes * height, cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(tmp, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    YAS_TRY_CUDA(e);
    return YAS_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ fusion
// Grows the map to at least `want_slots` (power of two) slots and `want_blocks`
// pool blocks; blocks keep their pool indices and contents, the table is
// rebuilt.  The sticky error bits of earlier calls are kept.
// Exchanges everything MapStruct::Swap exchanges (VoxelMap.cu:173-199): the
// device storage, its configuration, the intrinsics and the hibernation state.
// Pose and active flag stay with the handle.  Both streams must be idle.
static void swap_storage(yas_map *a, yas_map *b) {
    std::swap(a->cfg, b->cfg);
    std::swap(a->cam_K, b->cam_K);
    std::swap(a->slots, b->slots);
    std::swap(a->slot_mask, b->slot_mask);
    std::swap(a->block_keys, b->block_keys);
    std::swap(a->voxels, b->voxels);
    std::swap(a->visible, b->visible);
    std::swap(a->hdr, b->hdr);
    std::swap(a->hibernated, b->hibernated);
    std::swap(a->hib_slots, b->hib_slots);
    std::swap(a->hib_keys, b->hib_keys);
    std::swap(a->hib_voxels, b->hib_voxels);
    std::swap(a->hib_visible, b->hib_visible);
    std::swap(a->hib_hdr, b->hib_hdr);
}

static int map_grow(yas_map *m, long long want_slots, long long want_blocks) {
    YAS_TRY(read_header(m));
    const unsigned n = std::min(m->hdr_host->n_alloc, (unsigned)m->cfg.max_blocks);
    const unsigned old_bits = m->hdr_host->err_bits;
    long long ns = m->cfg.hash_slots;
    while (ns < want_slots) ns <<= 1;
    const long long nb = std::max<long long>(m->cfg.max_blocks, want_blocks);
    if (ns == m->cfg.hash_slots && nb == m->cfg.max_blocks) return YAS_OK;
    if (ns > (1LL << 30) || nb > (1LL << 30)) return YAS_ERR_CAPACITY;
    const size_t vb = m->cfg.voxel_format == YAS_VOXEL_F32 ? 8 : 4;
    HashSlot *slots = nullptr;
    unsigned long long *keys = nullptr;
    void *voxels = nullptr;
    int *visible = nullptr;
    if (cudaMalloc(&slots, (size_t)ns * sizeof(HashSlot)) != cudaSuccess ||
        cudaMalloc(&keys, (size_t)nb * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&voxels, (size_t)nb * kBlockVoxels * vb) != cudaSuccess ||
        cudaMalloc(&visible, (size_t)nb * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(slots);
        cudaFree(keys);
        cudaFree(voxels);
        cudaFree(visible);
        return YAS_ERR_OOM;
    }
    YAS_TRY_CUDA(cudaMemsetAsync(slots, 0xff, (size_t)ns * sizeof(HashSlot), m->stream));
    YAS_TRY_CUDA(cudaMemcpyAsync(keys, m->block_keys, (size_t)n * sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                                 m->stream));
    YAS_TRY_CUDA(cudaMemcpyAsync(voxels, m->voxels, (size_t)n * kBlockVoxels * vb, cudaMemcpyDeviceToDevice, m->stream));
    // pool indices do not move, so the visible list stays valid as it is
    const unsigned nv = std::min(m->hdr_host->n_visible, (unsigned)m->cfg.max_blocks);
    if (nv)
        YAS_TRY_CUDA(cudaMemcpyAsync(visible, m->visible, (size_t)nv * sizeof(int), cudaMemcpyDeviceToDevice, m->stream));
    YAS_TRY_CUDA(cudaMemsetAsync(&m->hdr->err_bits, 0, sizeof(unsigned), m->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));
    cudaFree(m->slots);
    cudaFree(m->block_keys);
    cudaFree(m->voxels);
    cudaFree(m->visible);
    m->slots = slots;
    m->block_keys = keys;
    m->voxels = voxels;
    m->visible = visible;
    m->cfg.hash_slots = (int)ns;
    m->cfg.max_blocks = (int)nb;
    m->slot_mask = (unsigned)(ns - 1);
    launch_rehash(map_view(m), n, m->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    YAS_TRY(read_header(m));
    const bool full = (m->hdr_host->err_bits & err_bit(YAS_ERR_TABLE_FULL)) != 0;
    const unsigned bits = old_bits | m->hdr_host->err_bits;
    YAS_TRY_CUDA(cudaMemcpyAsync(&m->hdr->err_bits, &bits, sizeof(unsigned), cudaMemcpyHostToDevice, m->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));
    return full ? YAS_ERR_TABLE_FULL : YAS_OK;
}

extern "C" {

YAS_API int yas_map_reserve(yas_map *m, int hash_slots, int max_blocks) {
    if (!m || hash_slots <= 0 || max_blocks <= 0) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    return map_grow(m, hash_slots, max_blocks);
}

YAS_API int yas_map_swap(yas_map *a, yas_map *b) {
    if (!a || !b) return YAS_ERR_BAD_ARG;
    if (a == b) return YAS_OK;
    YAS_TRY_CUDA(cudaStreamSynchronize(a->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(b->stream));
    swap_storage(a, b);
    return YAS_OK;
}

YAS_API int yas_map_fuse_map(yas_map *dst, yas_map *src) {
    if (!dst || !src || dst == src) return YAS_ERR_BAD_ARG;
    if (dst->hibernated || src->hibernated) return YAS_ERR_STATE;
    if (dst->cfg.voxel_format != src->cfg.voxel_format || dst->cfg.voxel_size != src->cfg.voxel_size)
        return YAS_ERR_BAD_ARG;
    YAS_TRY(read_header(src));
    YAS_TRY(read_header(dst));
    const unsigned nsrc = std::min(src->hdr_host->n_alloc, (unsigned)src->cfg.max_blocks);
    const unsigned ndst = std::min(dst->hdr_host->n_alloc, (unsigned)dst->cfg.max_blocks);
    if (nsrc == 0) return YAS_OK;
    if (ndst == 0) {
        // Swap: the destination takes the source's storage, configuration and
        // pose; the source is left with the empty storage.
        swap_storage(dst, src);
        std::scoped_lock lk(dst->pose_mutex, src->pose_mutex);
        std::swap(dst->Tcw, src->Tcw);
        return YAS_OK;
    }
    Pose64 Td, Ts;
    {
        std::scoped_lock lk(dst->pose_mutex, src->pose_mutex);
        Td = dst->Tcw;
        Ts = src->Tcw;
    }
    const Rigid32 T_src_dst = rigid_from(pose_mul(pose_inverse(Td), Ts));
    const Rigid32 T_dst_src = rigid_from(pose_mul(pose_inverse(Ts), Td));
    // room for the source's blocks in the destination (the reference reserves
    // both maps' capacities), grown again if they spread over more blocks
    long long want_blocks = (long long)ndst + 2LL * nsrc;
    YAS_TRY(map_grow(dst, 2 * want_blocks, want_blocks));
    YAS_TRY_CUDA(cudaMemsetAsync(&dst->hdr->err_bits, 0, sizeof(unsigned), dst->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(src->stream));
    for (int attempt = 0;; ++attempt) {
        launch_fuse_alloc(map_view(dst), map_view(src), dst->cfg.voxel_format, T_src_dst, nsrc, dst->stream);
        YAS_TRY_CUDA(cudaGetLastError());
        YAS_TRY(read_header(dst));
        const unsigned e = dst->hdr_host->err_bits;
        if (e & err_bit(YAS_ERR_COORD_RANGE)) return YAS_ERR_COORD_RANGE;
        if (!(e & (err_bit(YAS_ERR_POOL_FULL) | err_bit(YAS_ERR_TABLE_FULL)))) break;
        if (attempt == 3) return (e & err_bit(YAS_ERR_POOL_FULL)) ? YAS_ERR_POOL_FULL : YAS_ERR_TABLE_FULL;
        // keys claimed without a pool block are dropped by the rebuild; the
        // next pass inserts them again
        if (dst->hdr_host->n_alloc > (unsigned)dst->cfg.max_blocks) {
            const unsigned cap = (unsigned)dst->cfg.max_blocks;
            YAS_TRY_CUDA(cudaMemcpyAsync(&dst->hdr->n_alloc, &cap, sizeof(unsigned), cudaMemcpyHostToDevice,
                                         dst->stream));
        }
        YAS_TRY_CUDA(cudaMemsetAsync(&dst->hdr->err_bits, 0, sizeof(unsigned), dst->stream));
        want_blocks *= 2;
        YAS_TRY(map_grow(dst, 2 * want_blocks, want_blocks));
    }
    launch_fuse_blend(map_view(dst), map_view(src), dst->cfg.voxel_format, T_dst_src, dst->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    YAS_TRY_CUDA(cudaStreamSynchronize(dst->stream));
    // the reference releases the source's storage; here it is emptied and its
    // handle stays valid until yas_map_destroy
    return yas_map_reset(src);
}

YAS_API int yas_map_defuse_depth(yas_map *m, const float *depth, int width, int height, int pitch_bytes,
                                 int on_device, const yas_pose *Tcm) {
    if (!m || !depth || !Tcm || width <= 0 || height <= 0 || pitch_bytes < width * 4 || (pitch_bytes & 3))
        return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    const float *d = depth;
    if (!on_device) {
        MapExtra *ex = map_extra(m);
        YAS_TRY(ex->depth.ensure((size_t)pitch_bytes * height));
        YAS_TRY_CUDA(cudaMemcpyAsync(ex->depth.ptr, depth, (size_t)pitch_bytes * height, cudaMemcpyHostToDevice,
                                     m->stream));
        d = (const float *)ex->depth.ptr;
    }
    PosePair pp = make_pair(Tcm);
    YAS_TRY_CUDA(cudaMemcpyAsync(m->pose_dev, &pp, sizeof(pp), cudaMemcpyHostToDevice, m->stream));
    Cam cam = make_cam(m->cam_K.fx, m->cam_K.fy, m->cam_K.cx, m->cam_K.cy, width, height);
    MapDev v = map_view(m);
    YAS_TRY_CUDA(cudaMemsetAsync(&m->hdr->n_visible, 0, sizeof(unsigned), m->stream));
    launch_visible(v, cam, m->pose_dev, nullptr, m->stream);
    launch_deintegrate(v, m->cfg.voxel_format, d, pitch_bytes / 4, cam, m->pose_dev, m->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    if (!on_device) YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));
    return YAS_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ raycaster
YAS_API int yas_raycaster_create(yas_raycaster **out, int width, int height, const yas_intrinsics *K, void *stream) {
    if (!out || !K || width <= 0 || height <= 0) return YAS_ERR_BAD_ARG;
    *out = nullptr;
    yas_raycaster *rc = new yas_raycaster();
    rc->w = width;
    rc->h = height;
    rc->cam = make_cam(K->fx, K->fy, K->cx, K->cy, width, height);
    rc->stream = (cudaStream_t)stream;
    rc->rb.w = width;
    rc->rb.h = height;
    rc->rb.zw = (width + 7) / 8;
    rc->rb.zh = (height + 7) / 8;
    const size_t nz = (size_t)rc->rb.zw * rc->rb.zh;
    rc->rb.fw = (width + (1 << kFineShift) - 1) >> kFineShift;
    rc->rb.fh = (height + (1 << kFineShift) - 1) >> kFineShift;
    if (cudaMalloc(&rc->rb.znear, nz * 4) != cudaSuccess || cudaMalloc(&rc->rb.zfar, nz * 4) != cudaSuccess ||
        cudaMalloc(&rc->rb.queue, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&rc->rb.fnear, (size_t)rc->rb.fw * rc->rb.fh * 4) != cudaSuccess ||
        cudaMalloc(&rc->vmap, (size_t)width * height * 16) != cudaSuccess ||
        cudaMalloc(&rc->depth_tmp, (size_t)width * height * 4) != cudaSuccess ||
        cudaMalloc(&rc->pose_dev, sizeof(PosePair)) != cudaSuccess) {
        cudaGetLastError();
        yas_raycaster_destroy(rc);
        return YAS_ERR_OOM;
    }
    // the zero fill runs on the legacy stream, which the raycaster's
    // non-blocking stream does not wait for
    if (cudaMemset(rc->vmap, 0, (size_t)width * height * 16) != cudaSuccess ||
        cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess) {
        yas_raycaster_destroy(rc);
        return YAS_ERR_CUDA;
    }
    *out = rc;
    return YAS_OK;
}

YAS_API int yas_raycaster_destroy(yas_raycaster *rc) {
    if (!rc) return YAS_ERR_BAD_ARG;
    cudaStreamSynchronize(rc->stream);
    cudaFree(rc->rb.znear);
    cudaFree(rc->rb.zfar);
    cudaFree(rc->rb.queue);
    cudaFree(rc->rb.fnear);
    cudaFree(rc->vmap);
    cudaFree(rc->depth_tmp);
    cudaFree(rc->pose_dev);
    delete rc;
    return YAS_OK;
}

YAS_API int yas_raycaster_raycast(yas_raycaster *rc, yas_map *m, const yas_pose *Tcm) {
    if (!rc || !m || !Tcm) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    PosePair pp = make_pair(Tcm);
    cudaStream_t s = rc->stream;
    // The map's stream may differ: order the map's pending work first.
    if (m->stream != s) YAS_TRY_CUDA(cudaStreamSynchronize(m->stream));
    YAS_TRY_CUDA(cudaMemcpyAsync(rc->pose_dev, &pp, sizeof(pp), cudaMemcpyHostToDevice, s));
    YAS_TRY_CUDA(cudaMemsetAsync(&m->hdr->n_visible, 0, sizeof(unsigned), s));
    MapDev v = map_view(m);
    Cam vis_cam = make_cam(m->cam_K.fx, m->cam_K.fy, m->cam_K.cx, m->cam_K.cy, rc->w, rc->h);
    launch_visible(v, vis_cam, rc->pose_dev, nullptr, s);
    launch_zrange(v, rc->cam, rc->pose_dev, rc->rb, nullptr, s);
    launch_march(v, m->cfg.voxel_format, rc->cam, rc->pose_dev, rc->rb, rc->vmap, rc->w, nullptr, s);
    YAS_TRY_CUDA(cudaGetLastError());
    YAS_TRY_CUDA(cudaStreamSynchronize(s));
    MapHeader h;
    YAS_TRY_CUDA(cudaMemcpy(&h, m->hdr, sizeof(h), cudaMemcpyDeviceToHost));
    rc->last_visible = h.n_visible;
    return YAS_OK;
}

YAS_API int yas_raycaster_vmap(yas_raycaster *rc, const float **dev_vmap, int *pitch_bytes) {
    if (!rc || !dev_vmap) return YAS_ERR_BAD_ARG;
    *dev_vmap = reinterpret_cast<const float *>(rc->vmap);
    if (pitch_bytes) *pitch_bytes = rc->w * 16;
    return YAS_OK;
}

YAS_API int yas_raycaster_depth(yas_raycaster *rc, float *depth, int pitch_bytes, int on_device) {
    if (!rc || !depth || pitch_bytes < rc->w * 4 || (pitch_bytes & 3)) return YAS_ERR_BAD_ARG;
    if (on_device) {
        launch_vmap_to_depth(rc->vmap, rc->w, depth, pitch_bytes / 4, rc->w, rc->h, rc->stream);
        YAS_TRY_CUDA(cudaGetLastError());
        return YAS_OK;
    }
    launch_vmap_to_depth(rc->vmap, rc->w, rc->depth_tmp, rc->w, rc->w, rc->h, rc->stream);
    YAS_TRY_CUDA(cudaMemcpy2DAsync(depth, pitch_bytes, rc->depth_tmp, rc->w * 4, rc->w * 4, rc->h,
                                   cudaMemcpyDeviceToHost, rc->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(rc->stream));
    return YAS_OK;
}

YAS_API int yas_raycaster_num_visible(yas_raycaster *rc, unsigned *out) {
    if (!rc || !out) return YAS_ERR_BAD_ARG;
    *out = rc->last_visible;
    return YAS_OK;
}

YAS_API int yas_raycaster_num_rendering_blocks(yas_raycaster *rc, unsigned *out) {
    (void)rc;
    if (!rc || !out) return YAS_ERR_BAD_ARG;
    *out = 0;
    return YAS_OK;
}

YAS_API int yas_raycaster_zrange(yas_raycaster *rc, float *znear, float *zfar) {
    if (!rc || !znear || !zfar) return YAS_ERR_BAD_ARG;
    const size_t n = (size_t)rc->rb.zw * rc->rb.zh * 4;
    YAS_TRY_CUDA(cudaMemcpyAsync(znear, rc->rb.znear, n, cudaMemcpyDeviceToHost, rc->stream));
    YAS_TRY_CUDA(cudaMemcpyAsync(zfar, rc->rb.zfar, n, cudaMemcpyDeviceToHost, rc->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(rc->stream));
    return YAS_OK;
}

// ------------------------------------------------------------------ mesher
YAS_API int yas_mesher_create(yas_mesher **out, int max_triangles, void *stream) {
    if (!out || max_triangles <= 0) return YAS_ERR_BAD_ARG;
    *out = nullptr;
    yas_mesher *me = new yas_mesher();
    me->stream = (cudaStream_t)stream;
    me->mb.max_tris = max_triangles;
    const size_t t = (size_t)max_triangles;
    if (cudaMalloc(&me->mb.points, t * 36) != cudaSuccess || cudaMalloc(&me->mb.normals, t * 36) != cudaSuccess ||
        cudaMalloc(&me->mb.cases, t * 4) != cudaSuccess || cudaMalloc(&me->mb.cube_xyz, t * 12) != cudaSuccess ||
        cudaMalloc(&me->mb.counters, 64) != cudaSuccess) {
        cudaGetLastError();
        yas_mesher_destroy(me);
        return YAS_ERR_OOM;
    }
    mesh_tables_upload();
    *out = me;
    return YAS_OK;
}

YAS_API int yas_mesher_destroy(yas_mesher *me) {
    if (!me) return YAS_ERR_BAD_ARG;
    cudaStreamSynchronize(me->stream);
    cudaFree(me->mb.points);
    cudaFree(me->mb.normals);
    cudaFree(me->mb.cases);
    cudaFree(me->mb.cube_xyz);
    cudaFree(me->mb.counters);
    cudaFree(me->mb.block_tris);
    cudaFree(me->mb.block_offset);
    delete me;
    return YAS_OK;
}

YAS_API int yas_mesher_meshify(yas_mesher *me, yas_map *m, unsigned *out_num) {
    if (!me || !m) return YAS_ERR_BAD_ARG;
    if (m->hibernated) return YAS_ERR_STATE;
    unsigned n;
    YAS_TRY(yas_map_num_allocated(m, &n));
    YAS_TRY(launch_meshify(map_view(m), m->cfg.voxel_format, me->mb, n, me->stream));
    YAS_TRY_CUDA(cudaGetLastError());
    unsigned total = 0;
    YAS_TRY_CUDA(cudaMemcpyAsync(&total, me->mb.counters, 4, cudaMemcpyDeviceToHost, me->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(me->stream));
    const unsigned kept = total < (unsigned)me->mb.max_tris ? total : (unsigned)me->mb.max_tris;
    me->last_tris = kept;
    if (out_num) *out_num = kept;
    return total > (unsigned)me->mb.max_tris ? YAS_ERR_MESH_OVERFLOW : YAS_OK;
}

YAS_API int yas_mesher_copy(yas_mesher *me, float *points, float *normals, unsigned capacity) {
    if (!me) return YAS_ERR_BAD_ARG;
    if (capacity < me->last_tris) return YAS_ERR_CAPACITY;
    const size_t b = (size_t)me->last_tris * 36;
    if (b == 0) return YAS_OK;
    if (points) YAS_TRY_CUDA(cudaMemcpyAsync(points, me->mb.points, b, cudaMemcpyDeviceToHost, me->stream));
    if (normals) YAS_TRY_CUDA(cudaMemcpyAsync(normals, me->mb.normals, b, cudaMemcpyDeviceToHost, me->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(me->stream));
    return YAS_OK;
}

YAS_API int yas_mesher_copy_cases(yas_mesher *me, int *cases, int *cube_xyz, unsigned capacity) {
    if (!me) return YAS_ERR_BAD_ARG;
    if (capacity < me->last_tris) return YAS_ERR_CAPACITY;
    const size_t n = me->last_tris;
    if (n == 0) return YAS_OK;
    if (cases) YAS_TRY_CUDA(cudaMemcpyAsync(cases, me->mb.cases, n * 4, cudaMemcpyDeviceToHost, me->stream));
    if (cube_xyz) YAS_TRY_CUDA(cudaMemcpyAsync(cube_xyz, me->mb.cube_xyz, n * 12, cudaMemcpyDeviceToHost, me->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(me->stream));
    return YAS_OK;
}

// ------------------------------------------------------------------ tracker
YAS_API int yas_tracker_create(yas_tracker **out, int width, int height, const double *K, int num_levels,
                               const int *iterations, int mode, void *stream) {
    if (!out || !K || width <= 0 || height <= 0 || num_levels < 1 || num_levels > kMaxLevels ||
        (mode != YAS_TRACK_RGB && mode != YAS_TRACK_ICP && mode != YAS_TRACK_RGBD))
        return YAS_ERR_BAD_ARG;
    *out = nullptr;
    yas_tracker *tr = new yas_tracker();
    tr->w = width;
    tr->h = height;
    tr->L = num_levels;
    tr->mode = mode;
    tr->stream = (cudaStream_t)stream;
    for (int i = 0; i < 9; ++i) tr->K[i] = K[i];
    const int def_iters[kMaxLevels] = {10, 5, 3, 3, 3};
    for (int l = 0; l < kMaxLevels; ++l) {
        tr->iters[l] = iterations ? (l < num_levels ? iterations[l] : 0) : def_iters[l];
        const double s = (double)(1 << l);
        const double fx = K[0] / s, fy = K[4] / s, cx = K[2] / s, cy = K[5] / s;
        tr->dK[l][0] = fx;
        tr->dK[l][1] = fy;
        tr->dK[l][2] = cx;
        tr->dK[l][3] = cy;
        LevelCam &c = tr->cam[l];
        c.fx = (float)fx;
        c.fy = (float)fy;
        c.cx = (float)cx;
        c.cy = (float)cy;
        c.invfx = (float)(1.0 / fx);
        c.invfy = (float)(1.0 / fy);
        c.w = width >> l;
        c.h = height >> l;
        if (l < num_levels && (c.w < 4 || c.h < 4)) {
            delete tr;
            return YAS_ERR_BAD_ARG;
        }
    }
    tr->angle_th = sinf(20.f * 3.14159254f / 180.f);
    tr->dist_th = 0.01f;
    int st = tracker_alloc(tr);
    if (st != YAS_OK) {
        tracker_free(tr);
        delete tr;
        return st;
    }
    launch_gn_init(tr, pose_identity(), tr->stream);
    cudaError_t e = cudaStreamSynchronize(tr->stream);
    if (e != cudaSuccess) {
        record_cuda_error(e, "tracker init", __FILE__, __LINE__);
        tracker_free(tr);
        delete tr;
        return YAS_ERR_CUDA;
    }
    *out = tr;
    return YAS_OK;
}

YAS_API int yas_tracker_destroy(yas_tracker *tr) {
    if (!tr) return YAS_ERR_BAD_ARG;
    cudaStreamSynchronize(tr->stream);
    tracker_free(tr);
    delete tr;
    return YAS_OK;
}

static int stage_input(yas_tracker *tr, const void *src, int pitch, int row_bytes, int on_device,
                       const void **dev, int *dev_pitch) {
    if (on_device) {
        *dev = src;
        *dev_pitch = pitch;
        return YAS_OK;
    }
    YAS_TRY_CUDA(cudaMemcpy2DAsync(tr->staging, row_bytes, src, pitch, row_bytes, tr->h, cudaMemcpyHostToDevice,
                                   tr->stream));
    *dev = tr->staging;
    *dev_pitch = row_bytes;
    return YAS_OK;
}

static int tracker_set_image(yas_tracker *tr, const uint8_t *gray, int pitch, int on_device, bool reference) {
    if (!tr || !gray || pitch < tr->w) return YAS_ERR_BAD_ARG;
    const void *d;
    int dp;
    YAS_TRY(stage_input(tr, gray, pitch, tr->w, on_device, &d, &dp));
    tracker_image(tr, (const uint8_t *)d, 1, dp, reference, tr->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    if (!on_device) YAS_TRY_CUDA(cudaStreamSynchronize(tr->stream));
    return YAS_OK;
}

static int tracker_set_depth(yas_tracker *tr, const float *depth, int pitch, int on_device, bool reference) {
    if (!tr || !depth || pitch < tr->w * 4 || (pitch & 3)) return YAS_ERR_BAD_ARG;
    const void *d;
    int dp;
    YAS_TRY(stage_input(tr, depth, pitch, tr->w * 4, on_device, &d, &dp));
    tracker_depth(tr, d, 0, dp, 1.0f, nullptr, reference, tr->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    if (!on_device) YAS_TRY_CUDA(cudaStreamSynchronize(tr->stream));
    return YAS_OK;
}

YAS_API int yas_tracker_set_reference_image(yas_tracker *tr, const uint8_t *g, int p, int d) {
    return tracker_set_image(tr, g, p, d, true);
}
YAS_API int yas_tracker_set_tracking_image(yas_tracker *tr, const uint8_t *g, int p, int d) {
    return tracker_set_image(tr, g, p, d, false);
}
YAS_API int yas_tracker_set_reference_depth(yas_tracker *tr, const float *z, int p, int d) {
    return tracker_set_depth(tr, z, p, d, true);
}
YAS_API int yas_tracker_set_tracking_depth(yas_tracker *tr, const float *z, int p, int d) {
    return tracker_set_depth(tr, z, p, d, false);
}

YAS_API int yas_tracker_set_reference_model(yas_tracker *tr, const float *dev_vmap, int pitch) {
    if (!tr || !dev_vmap || pitch < tr->w * 16) return YAS_ERR_BAD_ARG;
    YAS_TRY_CUDA(cudaMemcpy2DAsync(tr->refb(0).vmap, tr->w * 16, dev_vmap, pitch, tr->w * 16, tr->h,
                                   cudaMemcpyDeviceToDevice, tr->stream));
    tracker_model(tr, tr->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    return YAS_OK;
}

YAS_API int yas_tracker_get_transform(yas_tracker *tr, const yas_pose *init, int swap_buffer, yas_pose *out) {
    if (!tr || !out) return YAS_ERR_BAD_ARG;
    Pose64 p0 = init ? pose_from(*init) : pose_identity();
    launch_gn_init(tr, p0, tr->stream);
    launch_gn_schedule(tr, tr->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    YAS_TRY_CUDA(cudaMemcpyAsync(tr->state_host, tr->state, sizeof(GNState), cudaMemcpyDeviceToHost, tr->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(tr->stream));
    const GNState &st = *tr->state_host;
    if (st.failed) {
        tr->good = false;
        *out = pose_to(pose_identity());
        return st.failed == kFailTimeout ? YAS_ERR_TIMEOUT : YAS_ERR_NUMERIC;
    }
    yas_pose r;
    for (int i = 0; i < 12; ++i) r.m[i] = st.best[i];
    *out = r;
    tr->good = true;
    if (swap_buffer) tr->cur = 1 - tr->cur;
    return YAS_OK;
}

YAS_API int yas_tracker_swap_frame_buffer(yas_tracker *tr) {
    if (!tr) return YAS_ERR_BAD_ARG;
    tr->cur = 1 - tr->cur;
    return YAS_OK;
}

YAS_API int yas_tracker_set_schedule(yas_tracker *tr, int fused) {
    if (!tr) return YAS_ERR_BAD_ARG;
    tr->use_fused = fused != 0;
    return YAS_OK;
}

YAS_API int yas_tracker_set_reduction(yas_tracker *tr, int compensated) {
    if (!tr) return YAS_ERR_BAD_ARG;
    const unsigned plain = compensated ? 0u : 1u;
    YAS_TRY_CUDA(cudaMemcpyAsync(&tr->state->plain_sums, &plain, sizeof(plain), cudaMemcpyHostToDevice, tr->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(tr->stream));
    return YAS_OK;
}

YAS_API int yas_tracker_check_wait_limit(yas_tracker *tr, int *out_status) {
    if (!tr || !out_status) return YAS_ERR_BAD_ARG;
    if (gn_batch_capacity() < 2) return YAS_ERR_STATE;
    GNBatchItem *d_item = nullptr;
    unsigned short *d_map = nullptr;
    if (cudaMalloc(&d_item, sizeof(GNBatchItem)) != cudaSuccess ||
        cudaMalloc(&d_map, 2 * sizeof(unsigned short)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_item);
        return YAS_ERR_OOM;
    }
    // every index in range: the descriptor's chunks are those of two CTAs and
    // CTA 0 touches only its own; only the missing CTA's rows never arrive
    GNBatchItem it;
    gn_batch_item_ctas(tr, 0, 2, &it);
    cudaError_t e = cudaMemcpyAsync(d_item, &it, sizeof(it), cudaMemcpyHostToDevice, tr->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_map, 0, 2 * sizeof(unsigned short), tr->stream);
    if (e == cudaSuccess) {
        launch_gn_init(tr, pose_identity(), tr->stream);
        e = launch_gn_batch(d_item, d_map, 1, tr->stream, gn_batch_pix(&it, 1));
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(tr->state_host, tr->state, sizeof(GNState), cudaMemcpyDeviceToHost, tr->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(tr->stream);
    cudaFree(d_item);
    cudaFree(d_map);
    if (e != cudaSuccess) {
        record_cuda_error(e, "wait limit check", __FILE__, __LINE__);
        return YAS_ERR_CUDA;
    }
    const int failed = tr->state_host->failed;
    *out_status = failed == kFailTimeout ? YAS_ERR_TIMEOUT : (failed ? YAS_ERR_NUMERIC : YAS_OK);
    tr->good = false;
    return YAS_OK;
}

YAS_API int yas_tracker_is_good(yas_tracker *tr, int *out) {
    if (!tr || !out) return YAS_ERR_BAD_ARG;
    *out = tr->good ? 1 : 0;
    return YAS_OK;
}

}  // extern "C"

namespace yas {
void launch_gn_linearise(yas_tracker *tr, int l, cudaStream_t s);
}

extern "C" {

YAS_API int yas_tracker_compute_step(yas_tracker *tr, int level, const yas_pose *T, double *H, double *b,
                                     double *stats) {
    if (!tr || !T || level < 0 || level >= tr->L) return YAS_ERR_BAD_ARG;
    launch_gn_init(tr, pose_from(*T), tr->stream);
    launch_gn_linearise(tr, level, tr->stream);
    YAS_TRY_CUDA(cudaGetLastError());
    YAS_TRY_CUDA(cudaMemcpyAsync(tr->state_host, tr->state, sizeof(GNState), cudaMemcpyDeviceToHost, tr->stream));
    YAS_TRY_CUDA(cudaStreamSynchronize(tr->stream));
    const GNState &st = *tr->state_host;
    if (H)
        for (int i = 0; i < 36; ++i) H[i] = st.H[i];
    if (b)
        for (int i = 0; i < 6; ++i) b[i] = st.b[i];
    if (stats)
        for (int i = 0; i < 4; ++i) stats[i] = st.stats[i];
    return YAS_OK;
}

YAS_API int yas_tracker_last_solve(yas_tracker *tr, double *H, double *b, double *update, yas_pose *estimate) {
    if (!tr) return YAS_ERR_BAD_ARG;
    YAS_TRY_CUDA(cudaStreamSynchronize(tr->stream));
    YAS_TRY_CUDA(cudaMemcpy(tr->state_host, tr->state, sizeof(GNState), cudaMemcpyDeviceToHost));
    const GNState &st = *tr->state_host;
    if (H)
        for (int i = 0; i < 36; ++i) H[i] = st.H[i];
    if (b)
        for (int i = 0; i < 6; ++i) b[i] = st.b[i];
    if (update)
        for (int i = 0; i < 6; ++i) update[i] = st.last_update[i];
    if (estimate)
        for (int i = 0; i < 12; ++i) estimate->m[i] = st.est[i];
    return YAS_OK;
}

YAS_API int yas_tracker_level_buffer(yas_tracker *tr, int level, int which, const void **dev_ptr, int *width,
                                     int *height, int *pitch_bytes) {
    if (!tr || !dev_ptr || level < 0 || level >= tr->L || which < 0 || which > 9) return YAS_ERR_BAD_ARG;
    TrackLevelBufs &c = tr->curb(level), &r = tr->refb(level);
    const void *p = nullptr;
    int esz = 4;
    switch (which) {
        case 0: p = c.intensity; break;
        case 1: p = tr->gx[level]; break;
        case 2: p = tr->gy[level]; break;
        case 3: p = c.invd; break;
        case 4: p = c.vmap; esz = 16; break;
        case 5: p = c.nmap; esz = 16; break;
        case 6: p = r.intensity; break;
        case 7: p = r.invd; break;
        case 8: p = r.vmap; esz = 16; break;
        default: p = r.nmap; esz = 16; break;
    }
    *dev_ptr = p;
    if (width) *width = tr->cam[level].w;
    if (height) *height = tr->cam[level].h;
    if (pitch_bytes) *pitch_bytes = tr->cam[level].w * esz;
    return YAS_OK;
}

}  // extern "C"
