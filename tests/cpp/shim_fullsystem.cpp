// shim_fullsystem.cpp — FullSystem's dense calls written with the reference's
// own types (Sophus::SE3d, Eigen matrices, cv::Mat, cv::cuda::GpuMat) against
// include/yas_rgbdfusion.hpp compiled with YAS_SHIM_SOPHUS and
// YAS_SHIM_OPENCV, statement for statement as in
// FullSystem/src/Tracking.cpp:17-19 (engines), :139-155
// (StereoInitialization), :162-197 (TrackRGBD) and :617-622, :703-716
// (CreateNewKeyFrame's raycast depth and submap switch).  The tests compile it
// against small stand-in headers for those types (tests/cpp/standin/).
//
// usage: shim_fullsystem <frames.bin> <out.txt>
//   frames.bin: int32 width, height, n; float fx, fy, cx, cy; then per frame
//               width*height gray u8 and width*height depth float32 (metres).
//   out.txt:    one "key values..." line per result, doubles printed exactly.
#include <cstdint>
#include <cstdio>
#include <vector>

#include <Eigen/Core>
#include <opencv2/core.hpp>
#include <opencv2/core/cuda.hpp>
#include <sophus/se3.hpp>

#include "yas_rgbdfusion.hpp"

struct Frame {  // the members of FullSystem's Frame this path reads
    cv::Mat mImGray, mImDepth;
    Sophus::SE3d mTcw, mTcp;
};

static void print_pose(FILE *out, int i, int status, const Sophus::SE3d &T) {
    const Eigen::Matrix<double, 3, 4> M = T.matrix3x4();
    std::fprintf(out, "pose %d %d", i, status);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) std::fprintf(out, " %.17g", M(r, c));
    std::fprintf(out, "\n");
}

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s frames.bin out.txt\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[3];
    float k[4];
    if (std::fread(hdr, 4, 3, f) != 3 || std::fread(k, 4, 4, f) != 4) return 2;
    const int w = hdr[0], h = hdr[1], n = hdr[2];
    std::vector<cv::Mat> gray, depth;
    for (int i = 0; i < n; ++i) {
        cv::Mat g(h, w, CV_8UC1), d(h, w, CV_32FC1);
        if (std::fread(g.data, 1, (size_t)w * h, f) != (size_t)w * h ||
            std::fread(d.data, 4, (size_t)w * h, f) != (size_t)w * h)
            return 2;
        gray.push_back(g);
        depth.push_back(d);
    }
    std::fclose(f);
    FILE *out = std::fopen(argv[2], "w");
    if (!out) return 2;

    try {
        Eigen::Matrix3f calib = Eigen::Matrix3f::Identity();
        calib(0, 0) = k[0], calib(1, 1) = k[1], calib(0, 2) = k[2], calib(1, 2) = k[3];
        // Tracking::Tracking (Tracking.cpp:17-19)
        RGBDTracking *mpTracker = new RGBDTracking(w, h, calib.cast<double>(), true, true);
        MeshEngine *mpMeshEngine = new MeshEngine(1 << 21);
        RayTraceEngine *mpRayTraceEngine = new RayTraceEngine(w, h, calib);

        Frame mCurrentFrame, mLastFrame;
        cv::cuda::GpuMat mRawDepth;
        MapStruct *mpCurrentMapStruct = nullptr;
        for (int i = 0; i < n; ++i) {
            mCurrentFrame.mImGray = gray[i];
            mCurrentFrame.mImDepth = depth[i];
            int status = 0;
            if (i == 0) {
                // StereoInitialization (Tracking.cpp:139-155)
                mCurrentFrame.mTcw = Sophus::SE3d();
                mCurrentFrame.mTcp = Sophus::SE3d();
                mpCurrentMapStruct = new MapStruct(calib);
                mpCurrentMapStruct->SetMeshEngine(mpMeshEngine);
                mpCurrentMapStruct->SetRayTraceEngine(mpRayTraceEngine);
                mpCurrentMapStruct->create(5000, 4000, 4500, 0.01f, 0.03f);
                mpCurrentMapStruct->SetPose(mCurrentFrame.mTcw);
                mpTracker->SetReferenceImage(mCurrentFrame.mImGray);
                mpTracker->SetReferenceDepth(mCurrentFrame.mImDepth);
                mRawDepth.upload(mCurrentFrame.mImDepth);
                mpCurrentMapStruct->Fuse(mRawDepth, mCurrentFrame.mTcw);
            } else {
                // TrackRGBD (Tracking.cpp:162-197)
                Sophus::SE3d Tmw = mpCurrentMapStruct->mTcw;
                Sophus::SE3d Tcm = Tmw.inverse() * mLastFrame.mTcw;
                mpCurrentMapStruct->RayTrace(Tcm);
                auto vmap = mpCurrentMapStruct->GetRayTracingResult();
                mpTracker->SetReferenceModel(vmap);
                mpTracker->SetTrackingImage(mCurrentFrame.mImGray);
                mpTracker->SetTrackingDepth(mCurrentFrame.mImDepth);
                Sophus::SE3d DT = mpTracker->GetTransform(Sophus::SE3d(), true);
                if (DT.translation().norm() > 0.1) {
                    status = 7;
                } else {
                    mCurrentFrame.mTcw = mLastFrame.mTcw * DT.inverse();
                    mCurrentFrame.mTcp = mLastFrame.mTcp * DT.inverse();
                    mRawDepth.upload(mCurrentFrame.mImDepth);
                    mpCurrentMapStruct->Fuse(mRawDepth, mCurrentFrame.mTcp);
                }
            }
            print_pose(out, i, status, mCurrentFrame.mTcp);
            mLastFrame = mCurrentFrame;
        }
        std::fprintf(out, "good %d\n", mpTracker->IsTrackingGood() ? 1 : 0);

        // CreateNewKeyFrame (Tracking.cpp:617-622): the keyframe's depth is the
        // raycast of the current submap, downloaded by cv::Mat(GpuMat)
        mCurrentFrame.mImDepth = cv::Mat(mpCurrentMapStruct->GetRayTracingResultDepth());
        double dsum = 0;
        int dn = 0;
        for (int r = 0; r < mCurrentFrame.mImDepth.rows; ++r)
            for (int c = 0; c < mCurrentFrame.mImDepth.cols; ++c) {
                const float v = mCurrentFrame.mImDepth.ptr<float>(r)[c];
                if (v > 0) dsum += v, ++dn;
            }
        std::fprintf(out, "keyframe_depth %.17g %d\n", dsum, dn);

        // MapDrawer (MapDrawer.cpp:197-199): a mesh of the submap
        if (!mpCurrentMapStruct->mbHasMesh) mpCurrentMapStruct->GenerateMesh();
        std::fprintf(out, "mesh %d %d\n", mpCurrentMapStruct->N, mpCurrentMapStruct->mplPoint != nullptr ? 1 : 0);

        // submap switch (Tracking.cpp:703-716)
        mpCurrentMapStruct->SetActiveFlag(false);
        MapStruct *pOld = mpCurrentMapStruct;
        mpCurrentMapStruct = new MapStruct(calib);
        mpCurrentMapStruct->SetMeshEngine(mpMeshEngine);
        mpCurrentMapStruct->SetRayTraceEngine(mpRayTraceEngine);
        mpCurrentMapStruct->create(5000, 4000, 4500, 0.01f, 0.03f);
        mpCurrentMapStruct->SetPose(mCurrentFrame.mTcw);
        mpCurrentMapStruct->SetActiveFlag(true);
        const Eigen::Matrix4d P = mpCurrentMapStruct->GetPose().matrix();
        std::fprintf(out, "switch %d %d %.17g %.17g %.17g\n", pOld->isActive() ? 1 : 0,
                     mpCurrentMapStruct->isActive() ? 1 : 0, P(0, 3), P(1, 3), P(2, 3));
        delete pOld;
        delete mpCurrentMapStruct;
        delete mpTracker;
        delete mpMeshEngine;
        delete mpRayTraceEngine;
    } catch (const yas::shim::Error &e) {
        std::fprintf(out, "error %d\n", e.status);
        std::fclose(out);
        return 1;
    } catch (const std::exception &e) {
        std::fprintf(out, "exception %s\n", e.what());
        std::fclose(out);
        return 1;
    }
    std::fclose(out);
    return 0;
}
