/* yas_rgbdfusion.hpp — the RGBDFusion classes (MapStruct, RayTraceEngine,
 * MeshEngine, RGBDTracking) as a header-only C++17 layer over the C ABI in
 * yas.h, so that FullSystem-style host code keeps its class names, method
 * names and control flow and links against libyas_gb300 instead.
 *
 * Reference interfaces mirrored (paths relative to the reference project):
 *   MapStruct        RGBDFusion/include/VoxelMap.h:32-144
 *   RayTraceEngine   RGBDFusion/include/RayTraceEngine.h:11-49
 *   MeshEngine       RGBDFusion/include/MeshEngine.h:8-24
 *   RGBDTracking     RGBDFusion/include/RGBDTracking.h:9-107
 *   ImageProc        RGBDFusion/include/ImageProc.h:8-24 (free functions)
 *
 * Types.  The reference passes Sophus::SE3d, Eigen::Matrix3f/3d, cv::Mat and
 * cv::cuda::GpuMat.  This header uses small stand-ins by default:
 *   yas::shim::SE3d      rigid transform, double, row-major [R | t];
 *   yas::shim::Matrix3f / Matrix3d   3x3 with operator()(r, c);
 *   yas::shim::Image     a pitched image view, on the host or on the device,
 *                        optionally owning its memory (shared).
 * Define YAS_SHIM_SOPHUS before including to use Sophus::SE3d (and Eigen's
 * matrices) directly, and YAS_SHIM_OPENCV to add cv::Mat / cv::cuda::GpuMat
 * overloads of every image argument and to return GpuMats from
 * MapStruct::GetRayTracingResult / GetRayTracingResultDepth, as the reference
 * does.  The OpenCV branch expects the caller on the legacy default stream
 * (engines created with a NULL stream), as FullSystem is.
 *
 * Errors.  The reference exits the process on a CUDA error (SafeCall).  Here
 * every failing call throws yas::shim::Error, which carries the yas_status.
 * Two statuses are behaviour, not errors, as in the reference: a NaN solve in
 * GetTransform returns the identity and IsTrackingGood() turns false.
 *
 * Names.  The classes live in namespace yas::shim and are brought into the
 * global namespace (as the reference declares them) unless
 * YAS_SHIM_NO_GLOBAL_NAMES is defined.
 */
#pragma once

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "yas.h"

#ifdef YAS_SHIM_SOPHUS
#include <Eigen/Core>
#include <sophus/se3.hpp>
#endif
#ifdef YAS_SHIM_OPENCV
#include <opencv2/core.hpp>
#include <opencv2/core/cuda.hpp>
#endif

namespace yas {
namespace shim {

class Error : public std::runtime_error {
public:
    explicit Error(int status)
        : std::runtime_error(std::string("yas: ") + yas_status_string(status)), status(status) {}
    int status;
};

inline void check(int status) {
    if (status != YAS_OK) throw Error(status);
}

/* ------------------------------------------------------------------ types */

#ifdef YAS_SHIM_SOPHUS
using SE3d = Sophus::SE3d;
using Matrix3f = Eigen::Matrix3f;
using Matrix3d = Eigen::Matrix3d;
inline yas_pose to_pose(const SE3d &T) {
    yas_pose p;
    const Eigen::Matrix<double, 3, 4> M = T.matrix3x4();
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) p.m[r * 4 + c] = M(r, c);
    return p;
}
inline SE3d from_pose(const yas_pose &p) {
    Eigen::Matrix4d M = Eigen::Matrix4d::Identity();
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) M(r, c) = p.m[r * 4 + c];
    return SE3d(M);
}
inline double translation_norm(const SE3d &T) { return T.translation().norm(); }
#else
/* Rigid transform [R | t] in double precision. */
class SE3d {
public:
    SE3d() {
        std::memset(m, 0, sizeof(m));
        m[0] = m[5] = m[10] = 1.0;
    }
    static SE3d from_matrix3x4(const double *rowmajor12) {
        SE3d T;
        std::memcpy(T.m, rowmajor12, sizeof(T.m));
        return T;
    }
    SE3d operator*(const SE3d &o) const {
        SE3d r;
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j)
                r.m[i * 4 + j] = m[i * 4] * o.m[j] + m[i * 4 + 1] * o.m[4 + j] + m[i * 4 + 2] * o.m[8 + j];
            r.m[i * 4 + 3] = m[i * 4] * o.m[3] + m[i * 4 + 1] * o.m[7] + m[i * 4 + 2] * o.m[11] + m[i * 4 + 3];
        }
        return r;
    }
    SE3d inverse() const {
        SE3d r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.m[i * 4 + j] = m[j * 4 + i];
        for (int i = 0; i < 3; ++i)
            r.m[i * 4 + 3] = -(r.m[i * 4] * m[3] + r.m[i * 4 + 1] * m[7] + r.m[i * 4 + 2] * m[11]);
        return r;
    }
    double operator()(int r, int c) const { return r == 3 ? (c == 3 ? 1.0 : 0.0) : m[r * 4 + c]; }
    double m[12];
};
template <typename T>
struct Matrix3 {
    Matrix3() { std::memset(a, 0, sizeof(a)); }
    Matrix3(T fx, T fy, T cx, T cy) : Matrix3() {
        a[0] = fx, a[4] = fy, a[2] = cx, a[5] = cy, a[8] = T(1);
    }
    T &operator()(int r, int c) { return a[r * 3 + c]; }
    T operator()(int r, int c) const { return a[r * 3 + c]; }
    T a[9];
};
using Matrix3f = Matrix3<float>;
using Matrix3d = Matrix3<double>;
inline yas_pose to_pose(const SE3d &T) {
    yas_pose p;
    std::memcpy(p.m, T.m, sizeof(p.m));
    return p;
}
inline SE3d from_pose(const yas_pose &p) { return SE3d::from_matrix3x4(p.m); }
inline double translation_norm(const SE3d &T) {
    return std::sqrt(T.m[3] * T.m[3] + T.m[7] * T.m[7] + T.m[11] * T.m[11]);
}
#endif

template <typename M>
inline yas_intrinsics to_intrinsics(const M &K) {
    yas_intrinsics k;
    k.fx = (float)K(0, 0), k.fy = (float)K(1, 1), k.cx = (float)K(0, 2), k.cy = (float)K(1, 2);
    return k;
}

/* A pitched image: rows x cols elements of elem_bytes, row stride `step`
 * bytes, in host or device memory.  `owner` keeps owned memory alive across
 * copies (the reference's cv::Mat / GpuMat reference counting). */
struct Image {
    void *data = nullptr;
    size_t step = 0;
    int rows = 0, cols = 0, elem_bytes = 0;
    bool on_device = false;
    std::shared_ptr<void> owner;

    Image() = default;
    Image(const void *d, int rows_, int cols_, int elem, size_t step_, bool dev)
        : data(const_cast<void *>(d)), step(step_), rows(rows_), cols(cols_), elem_bytes(elem), on_device(dev) {}
    static Image host_owned(int rows, int cols, int elem) {
        Image im;
        auto buf = std::shared_ptr<std::vector<unsigned char>>(
            new std::vector<unsigned char>((size_t)rows * cols * elem));
        im.data = buf->data();
        im.owner = buf;
        im.rows = rows, im.cols = cols, im.elem_bytes = elem;
        im.step = (size_t)cols * elem;
        return im;
    }
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
    template <typename T>
    T *ptr(int r = 0) const {
        return reinterpret_cast<T *>(static_cast<unsigned char *>(data) + (size_t)r * step);
    }
};

#ifdef YAS_SHIM_OPENCV
inline Image view(const cv::Mat &m) {
    return Image(m.data, m.rows, m.cols, (int)m.elemSize(), m.step, false);
}
inline Image view(const cv::cuda::GpuMat &m) {
    return Image(m.data, m.rows, m.cols, (int)m.elemSize(), m.step, true);
}
#endif

class MapStruct;

/* ------------------------------------------------------------------ MeshEngine */

class MeshEngine {
public:
    explicit MeshEngine(int MaxNumTriangle) { check(yas_mesher_create(&handle_, MaxNumTriangle, nullptr)); }
    ~MeshEngine() {
        if (handle_) yas_mesher_destroy(handle_);
    }
    MeshEngine(const MeshEngine &) = delete;
    MeshEngine &operator=(const MeshEngine &) = delete;

    /* MeshEngine::Meshify (MeshEngine.cu:293-340): fills the map's mplPoint,
     * mplNormal (new float[N]) and N = 9 * triangles. */
    inline void Meshify(MapStruct *pMapStruct);
    yas_mesher *handle() const { return handle_; }

private:
    yas_mesher *handle_ = nullptr;
};

/* ------------------------------------------------------------------ RayTraceEngine */

class RayTraceEngine {
public:
    template <typename K3>
    RayTraceEngine(int w, int h, const K3 &K) : w_(w), h_(h) {
        const yas_intrinsics k = to_intrinsics(K);
        check(yas_raycaster_create(&handle_, w, h, &k, nullptr));
    }
    ~RayTraceEngine() {
        if (handle_) yas_raycaster_destroy(handle_);
    }
    RayTraceEngine(const RayTraceEngine &) = delete;
    RayTraceEngine &operator=(const RayTraceEngine &) = delete;

    inline void RayTrace(MapStruct *pMapStruct, const SE3d &Tcm);
    unsigned GetNumVisibleBlock() {
        unsigned n = 0;
        check(yas_raycaster_num_visible(handle_, &n));
        return n;
    }
    unsigned GetNumRenderingBlocks() {
        unsigned n = 0;
        check(yas_raycaster_num_rendering_blocks(handle_, &n));
        return n;
    }
    /* Device float4 vertex map, aliasing the engine's buffer: the next
     * raycast overwrites it (as the reference's GpuMat header does). */
    Image GetVMap() {
        const float *v = nullptr;
        int pitch = 0;
        check(yas_raycaster_vmap(handle_, &v, &pitch));
        return Image(v, h_, w_, 16, (size_t)pitch, true);
    }
    /* VMapToDepth of the last raycast, float metres (0 = miss), host memory. */
    Image GetDepth() {
        Image im = Image::host_owned(h_, w_, 4);
        check(yas_raycaster_depth(handle_, im.ptr<float>(), (int)im.step, 0));
        return im;
    }
    yas_raycaster *handle() const { return handle_; }

private:
    yas_raycaster *handle_ = nullptr;
    int w_, h_;
};

/* ------------------------------------------------------------------ MapStruct */

class MapStruct {
public:
    template <typename K3>
    explicit MapStruct(const K3 &K) : mK(to_intrinsics(K)), mnId(nNextId++) {}
    ~MapStruct() {
        DeleteMesh();
        Release();
    }
    MapStruct(const MapStruct &) = delete;
    MapStruct &operator=(const MapStruct &) = delete;

    /* create(hashTableSize, bucketSize, voxelBlockSize, voxelSize, truncationDist)
     * (VoxelMap.cu:60-81): FP32 storage, the reference's depth gates. */
    void create(int hashTableSize, int bucketSize, int voxelBlockSize, float voxelSize_, float truncationDist_) {
        Release();
        check(yas_map_create_ref(&handle_, hashTableSize, bucketSize, voxelBlockSize, voxelSize_, truncationDist_,
                                 &mK, nullptr));
        voxelSize = voxelSize_, truncationDist = truncationDist_;
        sync_pose_to_handle();
    }
    /* Explicit grid and storage format (F32 / F16 / S24 / S16). */
    void create(const yas_map_config &cfg) {
        Release();
        check(yas_map_create(&handle_, &cfg, &mK, nullptr));
        voxelSize = cfg.voxel_size, truncationDist = cfg.trunc_dist;
        sync_pose_to_handle();
    }

    SE3d GetPose() {
        if (handle_) {
            yas_pose p;
            check(yas_map_get_pose(handle_, &p));
            mTcw = from_pose(p);
        }
        return mTcw;
    }
    void SetPose(const SE3d &Tcw) {
        mTcw = Tcw;
        sync_pose_to_handle();
    }

    void SetMeshEngine(MeshEngine *pMeshEngine) { mpMeshEngine = pMeshEngine; }
    void SetRayTraceEngine(RayTraceEngine *pRayTraceEngine) { mpRayTraceEngine = pRayTraceEngine; }

    void Reset() { check(yas_map_reset(require())); }
    /* True once the storage is released or holds no block (a fused-away
     * source is left empty, as the reference releases it). */
    bool Empty() {
        if (!handle_) return true;
        int e = 0;
        check(yas_map_empty(handle_, &e));
        return e != 0;
    }
    void Release() {
        if (handle_) {
            yas_map_destroy(handle_);
            handle_ = nullptr;
        }
        mbInHibernation = false;
    }
    /* Swap (VoxelMap.cu:173-199): storage, grid, intrinsics, id and mesh
     * change hands; poses and active flags stay. */
    void Swap(MapStruct *other) {
        if (handle_ && other->handle_) {
            check(yas_map_swap(handle_, other->handle_));
        } else {
            // one side has no storage: the handles themselves change hands,
            // each keeping the pose of the object it now belongs to
            std::swap(handle_, other->handle_);
            sync_pose_to_handle();
            other->sync_pose_to_handle();
        }
        std::swap(voxelSize, other->voxelSize);
        std::swap(truncationDist, other->truncationDist);
        std::swap(mbInHibernation, other->mbInHibernation);
        std::swap(mnId, other->mnId);
        std::swap(mK, other->mK);
        std::swap(mbHasMesh, other->mbHasMesh);
        std::swap(mplPoint, other->mplPoint);
        std::swap(mplNormal, other->mplNormal);
        std::swap(N, other->N);
    }

    void ResetNumVisibleBlocks() { check(yas_map_reset_visible(require())); }
    unsigned GetNumVisibleBlocks() {
        unsigned n = 0;
        check(yas_map_num_visible(require(), &n));
        return n;
    }
    unsigned GetVisibleBlocks() { return GetNumVisibleBlocks(); }
    void ResetVisibleBlocks() { ResetNumVisibleBlocks(); }
    unsigned CheckNumVisibleBlocks(int cols, int rows, const SE3d &Tcm) {
        unsigned n = 0;
        const yas_pose p = to_pose(Tcm);
        check(yas_map_check_visible(require(), cols, rows, &p, &n));
        return n;
    }

    /* Fuse(MapStruct*) (VoxelMap.cu:398-444): src is left empty. */
    void Fuse(MapStruct *pMapStruct) { check(yas_map_fuse_map(require(), pMapStruct->require())); }
    /* Fuse(GpuMat depth, Tcm) (VoxelMap.cu:825-884): float metres, host or device. */
    void Fuse(const Image &depth, const SE3d &Tcm) {
        const yas_pose p = to_pose(Tcm);
        check(yas_map_fuse_depth(require(), static_cast<const float *>(depth.data), depth.cols, depth.rows,
                                 (int)depth.step, depth.on_device ? 1 : 0, &p));
    }
#ifdef YAS_SHIM_OPENCV
    void Fuse(const cv::cuda::GpuMat &depth, const SE3d &Tcm) { Fuse(view(depth), Tcm); }
    void Fuse(const cv::Mat &depth, const SE3d &Tcm) { Fuse(view(depth), Tcm); }
#endif

    void SaveToFile(const std::string &strFileName) { check(yas_map_save(require(), strFileName.c_str())); }
    void ReadFromFile(const std::string &strFileName) {
        check(yas_map_load(require(), strFileName.c_str()));
        GetPose();
    }
    /* Reserve(hSize, bSize, vSize) (VoxelMap.cu:479-515). */
    void Reserve(int hSize, int /*bSize*/, int vSize) {
        long long slots = 1;
        while (slots < hSize || slots < 2LL * vSize) slots <<= 1;
        check(yas_map_reserve(require(), (int)slots, vSize));
    }

    void Hibernate() {
        check(yas_map_hibernate(require()));
        mbInHibernation = true;
    }
    void ReActivate() {
        check(yas_map_reactivate(require()));
        mbInHibernation = false;
    }

    void SetActiveFlag(bool flag) { check(yas_map_set_active(require(), flag ? 1 : 0)); }
    bool isActive() {
        int a = 0;
        check(yas_map_is_active(require(), &a));
        return a != 0;
    }

    void GenerateMesh() {
        if (!mbHasMesh && mpMeshEngine && !mbInHibernation) {
            mpMeshEngine->Meshify(this);
            mbHasMesh = true;
        }
    }
    void DeleteMesh() {
        if (mbHasMesh) {
            N = 0;
            delete[] mplPoint;
            delete[] mplNormal;
            mplPoint = mplNormal = nullptr;
            mbHasMesh = false;
        }
    }

    void RayTrace(const SE3d &Tcm) {
        if (mpRayTraceEngine) mpRayTraceEngine->RayTrace(this, Tcm);
    }
#ifdef YAS_SHIM_OPENCV
    /* GetRayTracingResult() (VoxelMap.cu:976-979): a CV_32FC4 GpuMat header
     * aliasing the engine's vertex map; the next raycast overwrites it. */
    cv::cuda::GpuMat GetRayTracingResult() {
        if (!mpRayTraceEngine) return cv::cuda::GpuMat();
        const Image v = mpRayTraceEngine->GetVMap();
        return cv::cuda::GpuMat(v.rows, v.cols, CV_32FC4, v.data, v.step);
    }
    /* GetRayTracingResultDepth() (VoxelMap.cu:981-987): VMapToDepth of the
     * last raycast into a new CV_32FC1 device image. */
    cv::cuda::GpuMat GetRayTracingResultDepth() {
        if (!mpRayTraceEngine) return cv::cuda::GpuMat();
        const Image v = mpRayTraceEngine->GetVMap();
        cv::cuda::GpuMat d(v.rows, v.cols, CV_32FC1);
        check(yas_raycaster_depth(mpRayTraceEngine->handle(), d.ptr<float>(), (int)d.step, 1));
        return d;
    }
#else
    Image GetRayTracingResult() { return mpRayTraceEngine ? mpRayTraceEngine->GetVMap() : Image(); }
    Image GetRayTracingResultDepth() { return mpRayTraceEngine ? mpRayTraceEngine->GetDepth() : Image(); }
#endif

    yas_map *handle() const { return handle_; }
    yas_map *require() const {
        if (!handle_) throw Error(YAS_ERR_STATE);
        return handle_;
    }

    // public state of the reference class
    float *mplPoint = nullptr;
    float *mplNormal = nullptr;
    int N = 0;
    bool mbHasMesh = false;
    bool mbInHibernation = false;
    MeshEngine *mpMeshEngine = nullptr;
    RayTraceEngine *mpRayTraceEngine = nullptr;
    float voxelSize = 0.f, truncationDist = 0.f;
    yas_intrinsics mK;
    SE3d mTcw;  // mirror of the handle's pose, refreshed by GetPose / SetPose
    unsigned long mnId;
    static inline unsigned long nNextId = 0;

private:
    void sync_pose_to_handle() {
        if (handle_) {
            const yas_pose p = to_pose(mTcw);
            check(yas_map_set_pose(handle_, &p));
        }
    }
    yas_map *handle_ = nullptr;
};

inline void MeshEngine::Meshify(MapStruct *pMapStruct) {
    unsigned ntri = 0;
    check(yas_mesher_meshify(handle_, pMapStruct->require(), &ntri));
    float *pts = new float[(size_t)ntri * 9 + 1];
    float *nrm = new float[(size_t)ntri * 9 + 1];
    const int s = yas_mesher_copy(handle_, pts, nrm, ntri);
    if (s != YAS_OK) {
        delete[] pts;
        delete[] nrm;
        throw Error(s);
    }
    delete[] pMapStruct->mplPoint;
    delete[] pMapStruct->mplNormal;
    pMapStruct->mplPoint = pts;
    pMapStruct->mplNormal = nrm;
    pMapStruct->N = (int)(ntri * 9);
}

inline void RayTraceEngine::RayTrace(MapStruct *pMapStruct, const SE3d &Tcm) {
    const yas_pose p = to_pose(Tcm);
    check(yas_raycaster_raycast(handle_, pMapStruct->require(), &p));
}

/* ------------------------------------------------------------------ RGBDTracking */

class RGBDTracking {
public:
    static constexpr int kNumPyr = 5;  // NUM_PYR, RGBDTracking.h:7

    /* RGBDTracking(w, h, K, bRGB, bIcp) (RGBDTracking.cu:5-64): 5 levels with
     * {10, 5, 3, 3, 3} iterations; `num_levels` / `iterations` override them. */
    template <typename K3>
    RGBDTracking(int w, int h, const K3 &K, bool bRGB, bool bIcp, int num_levels = kNumPyr,
                 const int *iterations = nullptr)
        : w_(w), h_(h) {
        static const int kIters[kNumPyr] = {10, 5, 3, 3, 3};
        double Kd[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Kd[r * 3 + c] = (double)K(r, c);
        const int mode = (bRGB ? YAS_TRACK_RGB : 0) | (bIcp ? YAS_TRACK_ICP : 0);
        check(yas_tracker_create(&handle_, w, h, Kd, num_levels, iterations ? iterations : kIters, mode, nullptr));
    }
    ~RGBDTracking() {
        if (handle_) yas_tracker_destroy(handle_);
    }
    RGBDTracking(const RGBDTracking &) = delete;
    RGBDTracking &operator=(const RGBDTracking &) = delete;

    bool IsTrackingGood() const {
        int g = 0;
        check(yas_tracker_is_good(handle_, &g));
        return g != 0;
    }
    /* Gray CV_8U and depth CV_32F (metres) frames, host or device. */
    void SetReferenceImage(const Image &imGray) {
        check(yas_tracker_set_reference_image(handle_, static_cast<const uint8_t *>(imGray.data), (int)imGray.step,
                                              imGray.on_device));
    }
    void SetReferenceDepth(const Image &imDepth) {
        keep_raw_depth(imDepth);
        check(yas_tracker_set_reference_depth(handle_, static_cast<const float *>(imDepth.data), (int)imDepth.step,
                                              imDepth.on_device));
    }
    void SetTrackingImage(const Image &imGray) {
        check(yas_tracker_set_tracking_image(handle_, static_cast<const uint8_t *>(imGray.data), (int)imGray.step,
                                             imGray.on_device));
    }
    void SetTrackingDepth(const Image &imDepth) {
        keep_raw_depth(imDepth);
        check(yas_tracker_set_tracking_depth(handle_, static_cast<const float *>(imDepth.data), (int)imDepth.step,
                                             imDepth.on_device));
    }
    /* SetReferenceModel(GpuMat vmap): device float4. */
    void SetReferenceModel(const Image &vmap) {
        if (!vmap.on_device) throw Error(YAS_ERR_BAD_ARG);
        check(yas_tracker_set_reference_model(handle_, static_cast<const float *>(vmap.data), (int)vmap.step));
    }
#ifdef YAS_SHIM_OPENCV
    void SetReferenceImage(const cv::Mat &m) { SetReferenceImage(view(m)); }
    void SetReferenceDepth(const cv::Mat &m) { SetReferenceDepth(view(m)); }
    void SetTrackingImage(const cv::Mat &m) { SetTrackingImage(view(m)); }
    void SetTrackingDepth(const cv::Mat &m) { SetTrackingDepth(view(m)); }
    void SetReferenceModel(const cv::cuda::GpuMat &m) { SetReferenceModel(view(m)); }
#endif

    /* GetTransform(init, bSwapBuffer) (RGBDTracking.cu:152-214).  A NaN solve
     * returns the identity with IsTrackingGood() false, as the reference. */
    SE3d GetTransform(const SE3d &init, bool bSwapBuffer) {
        const yas_pose p0 = to_pose(init);
        yas_pose out;
        const int s = yas_tracker_get_transform(handle_, &p0, bSwapBuffer ? 1 : 0, &out);
        if (s == YAS_ERR_NUMERIC) return SE3d();
        check(s);
        return from_pose(out);
    }
    void SwapFrameBuffer() { check(yas_tracker_swap_frame_buffer(handle_)); }

    /* GetReferenceDepth (RGBDTracking.cu:547-550): the raw depth of the last
     * Set*Depth call (the reference returns its raw-depth upload buffer,
     * whatever the level argument).  Host memory, float metres. */
    Image GetReferenceDepth(int /*lvl*/ = 0) const { return raw_depth_; }

    /* WriteDebugImages (RGBDTracking.cu:557-568): level-0 current and
     * reference intensity and the current gradients, written as PFM
     * (portable float map) files curr_image.pfm, last_image.pfm, gx.pfm and
     * gy.pfm in `dir`. */
    void WriteDebugImages(const std::string &dir = ".") const {
        static const struct {
            int which;
            const char *name;
        } kOut[4] = {{0, "curr_image.pfm"}, {6, "last_image.pfm"}, {1, "gx.pfm"}, {2, "gy.pfm"}};
        for (const auto &o : kOut) {
            const void *p = nullptr;
            int w = 0, h = 0, pitch = 0;
            check(yas_tracker_level_buffer(handle_, 0, o.which, &p, &w, &h, &pitch));
            std::vector<float> img((size_t)w * h);
            check(yas_copy_to_host(img.data(), w * 4, p, pitch, w * 4, h));
            const std::string path = dir + "/" + o.name;
            FILE *f = std::fopen(path.c_str(), "wb");
            if (!f) throw Error(YAS_ERR_IO);
            std::fprintf(f, "Pf\n%d %d\n-1.0\n", w, h);
            // PFM rows run bottom to top
            bool ok = true;
            for (int r = h - 1; r >= 0; --r) ok = ok && std::fwrite(&img[(size_t)r * w], 4, w, f) == (size_t)w;
            ok = std::fclose(f) == 0 && ok;
            if (!ok) throw Error(YAS_ERR_IO);
        }
    }

    yas_tracker *handle() const { return handle_; }

private:
    void keep_raw_depth(const Image &d) {
        Image im = Image::host_owned(h_, w_, 4);
        check(yas_copy_to_host(im.data, (int)im.step, d.data, (int)d.step, w_ * 4, h_));
        raw_depth_ = im;
    }
    yas_tracker *handle_ = nullptr;
    int w_, h_;
    Image raw_depth_;
};

/* ------------------------------------------------------------------ ImageProc */
/* The free functions of ImageProc.h:8-24 on device images (GpuMat roles): the
 * output image must be allocated by the caller with the input's size (or the
 * pyramid level's, for PyrDownDepth); pixels the reference leaves unwritten
 * keep their contents. */

inline void require_device(const Image &a, int elem) {
    if (!a.on_device || a.empty() || a.elem_bytes != elem) throw Error(YAS_ERR_BAD_ARG);
}

inline void PyrDownDepth(const Image &src, Image &dst) {
    require_device(src, 4);
    require_device(dst, 4);
    check(yas_pyr_down_depth(static_cast<const float *>(src.data), src.cols, src.rows, (int)src.step,
                             static_cast<float *>(dst.data), dst.cols, dst.rows, (int)dst.step, nullptr));
}
inline void ComputeVertexMap(const Image &depth_inv, Image &vmap, float invfx, float invfy, float cx, float cy,
                             float cut_off) {
    require_device(depth_inv, 4);
    require_device(vmap, 16);
    check(yas_compute_vertex_map(static_cast<const float *>(depth_inv.data), depth_inv.cols, depth_inv.rows,
                                 (int)depth_inv.step, static_cast<float *>(vmap.data), (int)vmap.step, invfx, invfy, cx,
                                 cy, cut_off, nullptr));
}
inline void ComputeNormalMap(const Image &vmap, Image &nmap) {
    require_device(vmap, 16);
    require_device(nmap, 16);
    check(yas_compute_normal_map(static_cast<const float *>(vmap.data), vmap.cols, vmap.rows, (int)vmap.step,
                                 static_cast<float *>(nmap.data), (int)nmap.step, nullptr));
}
inline void DepthToInvDepth(const Image &depth, Image &depth_inv) {
    require_device(depth, 4);
    require_device(depth_inv, 4);
    check(yas_depth_to_inv_depth(static_cast<const float *>(depth.data), depth.cols, depth.rows, (int)depth.step,
                                 static_cast<float *>(depth_inv.data), (int)depth_inv.step, nullptr));
}
inline void ComputeImageGradientCentralDifference(const Image &image, Image &gx, Image &gy) {
    require_device(image, 4);
    require_device(gx, 4);
    require_device(gy, 4);
    if (gx.step != gy.step) throw Error(YAS_ERR_BAD_ARG);
    check(yas_image_gradient(static_cast<const float *>(image.data), image.cols, image.rows, (int)image.step,
                             static_cast<float *>(gx.data), static_cast<float *>(gy.data), (int)gx.step, nullptr));
}
template <typename K3>
inline void TransformReferencePoint(const Image &depth_inv, Image &vmap, const K3 &K, const SE3d &T) {
    require_device(depth_inv, 4);
    require_device(vmap, 16);
    double Kd[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Kd[r * 3 + c] = (double)K(r, c);
    const yas_pose p = to_pose(T);
    check(yas_transform_reference_point(static_cast<const float *>(depth_inv.data), depth_inv.cols, depth_inv.rows,
                                        (int)depth_inv.step, static_cast<float *>(vmap.data), (int)vmap.step, Kd, &p,
                                        nullptr));
}
inline void VMapToDepth(const Image &vmap, Image &depth) {
    require_device(vmap, 16);
    require_device(depth, 4);
    check(yas_vmap_to_depth(static_cast<const float *>(vmap.data), vmap.cols, vmap.rows, (int)vmap.step,
                            static_cast<float *>(depth.data), (int)depth.step, nullptr));
}

/* RenderScene(vmap, nmap, image) (ImageProc.cu:128-139): RGBA8 into `image`
 * (host or device, rows x cols of the vertex map). */
inline void RenderScene(const Image &vmap, const Image &nmap, Image &image) {
    if (!vmap.on_device || !nmap.on_device || vmap.step != nmap.step) throw Error(YAS_ERR_BAD_ARG);
    if (image.empty()) image = Image::host_owned(vmap.rows, vmap.cols, 4);
    check(yas_render_scene(static_cast<const float *>(vmap.data), static_cast<const float *>(nmap.data), vmap.cols,
                           vmap.rows, (int)vmap.step, nullptr, static_cast<uint8_t *>(image.data), (int)image.step,
                           image.on_device ? 1 : 0, nullptr));
}

}  // namespace shim
}  // namespace yas

#ifndef YAS_SHIM_NO_GLOBAL_NAMES
using yas::shim::MapStruct;
using yas::shim::MeshEngine;
using yas::shim::RayTraceEngine;
using yas::shim::ComputeImageGradientCentralDifference;
using yas::shim::ComputeNormalMap;
using yas::shim::ComputeVertexMap;
using yas::shim::DepthToInvDepth;
using yas::shim::PyrDownDepth;
using yas::shim::RenderScene;
using yas::shim::RGBDTracking;
using yas::shim::TransformReferencePoint;
using yas::shim::VMapToDepth;
#endif
