// shim_tracking.cpp — the dense calls of Tracking::StereoInitialization and
// Tracking::TrackRGBD (FullSystem/src/Tracking.cpp:139-197), and the MapStruct
// calls of MapDrawer / CreateNewKeyFrame, written against yas_rgbdfusion.hpp
// the way FullSystem writes them against RGBDFusion's classes.
//
// usage: shim_tracking <frames.bin> <out.txt> <work dir>
//   frames.bin: int32 width, height, n; float fx, fy, cx, cy; then per frame
//               width*height gray u8 and width*height depth float32 (metres).
//   out.txt:    one "key values..." line per result, doubles printed exactly.
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "yas_rgbdfusion.hpp"

using yas::shim::Image;
using yas::shim::Matrix3d;
using yas::shim::Matrix3f;
using yas::shim::SE3d;

static void print_pose(FILE *out, const char *key, int i, int status, const SE3d &T) {
    std::fprintf(out, "%s %d %d", key, i, status);
    for (int k = 0; k < 12; ++k) std::fprintf(out, " %.17g", T.m[k]);
    std::fprintf(out, "\n");
}

static double image_sum(const Image &im, int *count) {
    double s = 0;
    int c = 0;
    for (int r = 0; r < im.rows; ++r)
        for (int x = 0; x < im.cols; ++x) {
            const float v = im.ptr<float>(r)[x];
            if (v > 0) s += v, ++c;
        }
    if (count) *count = c;
    return s;
}

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s frames.bin out.txt workdir\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[3];
    float k[4];
    if (std::fread(hdr, 4, 3, f) != 3 || std::fread(k, 4, 4, f) != 4) return 2;
    const int W = hdr[0], H = hdr[1], n = hdr[2];
    std::vector<std::vector<uint8_t>> gray(n, std::vector<uint8_t>((size_t)W * H));
    std::vector<std::vector<float>> depth(n, std::vector<float>((size_t)W * H));
    for (int i = 0; i < n; ++i)
        if (std::fread(gray[i].data(), 1, gray[i].size(), f) != gray[i].size() ||
            std::fread(depth[i].data(), 4, depth[i].size(), f) != depth[i].size())
            return 2;
    std::fclose(f);
    FILE *out = std::fopen(argv[2], "w");
    if (!out) return 2;
    const std::string dir = argv[3];

    try {
        // Tracking::Tracking (Tracking.cpp:17-19), with the 3-level schedule
        const Matrix3f K(k[0], k[1], k[2], k[3]);
        const Matrix3d Kd(k[0], k[1], k[2], k[3]);
        const int iters[3] = {10, 5, 3};
        RGBDTracking tracker(W, H, Kd, true, true, 3, iters);
        MeshEngine mesher(1 << 21);
        RayTraceEngine raytracer(W, H, K);

        MapStruct ms(K);
        ms.create(1 << 18, 4000, 1 << 15, 0.008f, 0.024f);
        ms.SetMeshEngine(&mesher);
        ms.SetRayTraceEngine(&raytracer);
        ms.SetPose(SE3d());

        SE3d Tcp;  // camera in the submap
        for (int i = 0; i < n; ++i) {
            const Image g(gray[i].data(), H, W, 1, (size_t)W, false);
            const Image d(depth[i].data(), H, W, 4, (size_t)W * 4, false);
            int status = 0;
            if (i == 0) {
                // StereoInitialization (Tracking.cpp:140-155)
                tracker.SetReferenceImage(g);
                tracker.SetReferenceDepth(d);
                ms.Fuse(d, Tcp);
            } else {
                // TrackRGBD (Tracking.cpp:162-197); the submap sits at the origin,
                // so Tmw.inverse() * mLastFrame.mTcw is the last Tcp
                ms.RayTrace(Tcp);
                tracker.SetReferenceModel(ms.GetRayTracingResult());
                tracker.SetTrackingImage(g);
                tracker.SetTrackingDepth(d);
                const SE3d DT = tracker.GetTransform(SE3d(), true);
                if (yas::shim::translation_norm(DT) > 0.1) {
                    status = YAS_ERR_TRACK_LOST;
                } else {
                    Tcp = Tcp * DT.inverse();
                    ms.Fuse(d, Tcp);
                }
            }
            print_pose(out, "pose", i, status, Tcp);
        }
        std::fprintf(out, "good %d\n", tracker.IsTrackingGood() ? 1 : 0);
        std::fprintf(out, "visible %u\n", ms.GetNumVisibleBlocks());

        // CreateNewKeyFrame's raycast depth (Tracking.cpp:622)
        ms.RayTrace(Tcp);
        std::fprintf(out, "raytracer %u %u\n", raytracer.GetNumVisibleBlock(), raytracer.GetNumRenderingBlocks());
        int hits = 0;
        const double dsum = image_sum(ms.GetRayTracingResultDepth(), &hits);
        std::fprintf(out, "depth %.17g %d\n", dsum, hits);

        // MapDrawer (MapDrawer.cpp:197-210)
        ms.GenerateMesh();
        double psum = 0;
        for (int i = 0; i < ms.N; ++i) psum += ms.mplPoint[i];
        std::fprintf(out, "mesh %d %d %.17g\n", ms.N, ms.mbHasMesh ? 1 : 0, psum);
        ms.DeleteMesh();
        std::fprintf(out, "mesh_deleted %d %d\n", ms.N, ms.mbHasMesh ? 1 : 0);

        // Hibernate / ReActivate: the raycast afterwards is the same
        ms.Hibernate();
        const int hib = ms.mbInHibernation ? 1 : 0;
        ms.GenerateMesh();  // no-op while hibernated
        ms.ReActivate();
        ms.RayTrace(Tcp);
        int hits2 = 0;
        const double dsum2 = image_sum(ms.GetRayTracingResultDepth(), &hits2);
        std::fprintf(out, "hibernate %d %d %d %d\n", hib, ms.mbInHibernation ? 1 : 0, ms.mbHasMesh ? 1 : 0,
                     (dsum2 == dsum && hits2 == hits) ? 1 : 0);

        // SaveToFile / ReadFromFile, then Swap with a map without storage
        SE3d Tw;
        Tw.m[3] = 0.25, Tw.m[7] = -0.5, Tw.m[11] = 1.0;
        ms.SetPose(Tw);
        const std::string path = dir + "/submap.yas";
        ms.SaveToFile(path);
        MapStruct loaded(K);
        loaded.create(1 << 10, 4000, 64, 0.008f, 0.024f);
        loaded.ReadFromFile(path);
        unsigned na = 0, nb = 0;
        yas::shim::check(yas_map_num_allocated(ms.handle(), &na));
        yas::shim::check(yas_map_num_allocated(loaded.handle(), &nb));
        std::fprintf(out, "file %u %u %.17g\n", na, nb, loaded.mTcw.m[11]);
        MapStruct bare(K);
        const unsigned long id_loaded = loaded.mnId, id_bare = bare.mnId;
        bare.Swap(&loaded);
        std::fprintf(out, "swap %d %d %d\n", bare.Empty() ? 1 : 0, loaded.Empty() ? 1 : 0,
                     (bare.mnId == id_loaded && loaded.mnId == id_bare) ? 1 : 0);

        // Fuse(MapStruct*): the loaded copy folds back into an empty map
        MapStruct sink(K);
        sink.create(1 << 18, 4000, 1 << 15, 0.008f, 0.024f);
        sink.Fuse(&bare);
        unsigned ns = 0;
        yas::shim::check(yas_map_num_allocated(sink.handle(), &ns));
        std::fprintf(out, "fuse_map %u %d\n", ns, bare.Empty() ? 1 : 0);

        // RenderScene on the model maps of the last frame
        const void *vm = nullptr, *nm = nullptr;
        int lw = 0, lh = 0, vp = 0, np = 0;
        yas::shim::check(yas_tracker_level_buffer(tracker.handle(), 0, 8, &vm, &lw, &lh, &vp));
        yas::shim::check(yas_tracker_level_buffer(tracker.handle(), 0, 9, &nm, &lw, &lh, &np));
        Image rgba;
        RenderScene(Image(vm, lh, lw, 16, (size_t)vp, true), Image(nm, lh, lw, 16, (size_t)np, true), rgba);
        unsigned long long rsum = 0;
        for (int r = 0; r < rgba.rows; ++r)
            for (int x = 0; x < rgba.cols * 4; ++x) rsum += rgba.ptr<uint8_t>(r)[x];
        std::fprintf(out, "render %d %d %llu\n", rgba.cols, rgba.rows, rsum);

        // VMapToDepth (a free function) on the model vertex map, written into a
        // device image the library owns and the run no longer needs (the
        // tracker's level-0 inverse depth of the current frame)
        {
            const void *scratch = nullptr;
            int sw = 0, sh = 0, sp = 0;
            yas::shim::check(yas_tracker_level_buffer(tracker.handle(), 0, 3, &scratch, &sw, &sh, &sp));
            Image dimg(scratch, sh, sw, 4, (size_t)sp, true);
            VMapToDepth(Image(vm, lh, lw, 16, (size_t)vp, true), dimg);
            std::vector<float> a((size_t)lw * lh), v4((size_t)lw * lh * 4);
            yas::shim::check(yas_copy_to_host(a.data(), lw * 4, scratch, sp, lw * 4, lh));
            yas::shim::check(yas_copy_to_host(v4.data(), lw * 16, vm, vp, lw * 16, lh));
            int ok = 1;
            for (size_t i = 0; i < a.size(); ++i) {
                const float want = v4[4 * i + 3] > 0.0f ? v4[4 * i + 2] : 0.0f;
                if (a[i] != want) ok = 0;
            }
            std::fprintf(out, "vmap_to_depth %d\n", ok);
        }

        // GetReferenceDepth: the raw depth of the last Set*Depth call
        const Image raw = tracker.GetReferenceDepth();
        bool same = raw.rows == H && raw.cols == W;
        for (int r = 0; same && r < H; ++r)
            for (int x = 0; x < W; ++x)
                if (raw.ptr<float>(r)[x] != depth[n - 1][(size_t)r * W + x]) same = false;
        std::fprintf(out, "raw_depth %d\n", same ? 1 : 0);
        tracker.WriteDebugImages(dir);
        std::fprintf(out, "debug_images 1\n");

        // errors surface as exceptions carrying the status
        MapStruct never_created(K);
        int status = 0;
        try {
            never_created.Reset();
        } catch (const yas::shim::Error &e) {
            status = e.status;
        }
        std::fprintf(out, "error %d\n", status);
    } catch (const yas::shim::Error &e) {
        std::fprintf(out, "failed %d %s\n", e.status, e.what());
        std::fclose(out);
        return 1;
    }
    std::fclose(out);
    return 0;
}
