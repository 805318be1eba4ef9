// yas_track.h — tracker structures: per-level cameras, the device-resident
// Gauss-Newton state, and the tracker handle.
#pragma once

#include "yas_internal.h"

namespace yas {

constexpr int kMaxLevels = 5;
constexpr int kRedWidth = 32;       // values reduced per CTA (padded)
constexpr int kMaxCtas = 8192;      // partial-sum rows per pass
constexpr int kTrackThreads = 256;
constexpr int kPixPerThread = 1;

// Camera of one pyramid level: K / 2^l with K(2,2) = 1 (RGBDTracking.cu:16-26).
struct LevelCam {
    float fx, fy, cx, cy;
    float invfx, invfy;
    int w, h;
};

// GNState::failed values: a NaN update, or a bounded wait of the fused
// schedule that gave up.
constexpr int kFailNumeric = 1;
constexpr int kFailTimeout = 3;

// Gauss-Newton state, device resident; written only by the last CTA of a pass.
struct __align__(16) GNState {
    double est[12];         // current estimate T (reference frame -> current frame)
    double best[12];        // lastSuccessEstimate
    double last_error;      // per level, reset at the first iteration of a level
    int failed;             // NaN in the solve: estimate abandoned
    int n_iter;
    int n_success;
    int level_of_last;      // level of the last solve
    float Tf[12];           // float copy of est (row-major [R|t])
    float RKinv[kMaxLevels][9];  // float(R * K_l^-1) for TransformReferencePoint
    float huber_th;         // 4.685 * stddev of the photometric residuals
    float pad_f[3];
    double a_sums[kRedWidth];   // pass A totals: 0..26 ICP H|b, 27 ICP sum r^2, 28 ICP count,
                                // 29 RGB count, 30 RGB sum r, 31 RGB sum r^2
    double b_sums[kRedWidth];   // pass B totals: 0..26 RGB H|b, 27 RGB sum w r^2
    double H[36];           // last combined system
    double b[6];
    double stats[4];        // residualSum, numResidual, huber_th, icp count
    double last_update[6];
    unsigned epoch;         // launches of the fused schedule (row tags)
    unsigned abort_word;    // set when a bounded wait of the fused schedule gave up
    unsigned plain_sums;    // 1: plain FP32 totals (the reference's); 0: compensated totals
};

// One pyramid level of a fused Gauss-Newton schedule: camera, iterations,
// the pixel share of each CTA and the level maps.
struct FusedLevel {
    LevelCam c;
    int iters;
    int chunk;  // pixels per CTA (a multiple of 32)
    int pix;    // pixels per thread, ceil(chunk / threads per CTA)
    const float *ref_int, *ref_invd, *ref_z;
    const float4 *ref_vmap, *ref_nmap;
    const float *cur_int, *cur_gx, *cur_gy;
    const float4 *cur_vmap, *cur_nmap;
};

// One tracker's share of a batched Gauss-Newton launch: CTAs cta0 .. cta0 +
// nctas - 1 run its fused schedule over its own rows and state.
struct GNBatchItem {
    FusedLevel lv[kMaxLevels];
    int L, mode;
    float angle_th, dist_th;
    unsigned long long *rows;
    float4 *res4;
    GNState *st;
    int cta0, nctas;
};

struct TrackLevelBufs {
    float *intensity;
    float *invd;
    float *z;  // 1 / invd where invd > 0, else 0: the depth the photometric warp uses
    float4 *vmap;
    float4 *nmap;
};

void launch_image_level0(const uint8_t *src, int channels, int bgr, int pitch, int w, int h, float *inten,
                         float *gx, float *gy, cudaStream_t s);
void launch_image_level(const float *prev, int pw, int ph, int w, int h, float *inten, float *gx, float *gy,
                        cudaStream_t s);
void launch_depth_level0(const void *src, int is_u16, int pitch, float scale, const LevelCam &c,
                         float *depth_m, float *invd, float *zmap, float4 *vmap, float4 *nmap, cudaStream_t s);
void launch_depth_level(const float *prev, int pw, const LevelCam &c, float *invd, float *zmap, float4 *vmap,
                        float4 *nmap, cudaStream_t s);
void launch_model_pyramid(int L, const int *w, const int *h, float4 *const *vmap, float4 *const *nmap,
                          cudaStream_t s);
void launch_render_scene(const float4 *vmap, const float4 *nmap, int vpitch, int w, int h, float3 light,
                         uchar4 *out, int opitch, cudaStream_t s);

}  // namespace yas

struct yas_tracker {
    int w = 0, h = 0, L = 0, mode = YAS_TRACK_RGBD;
    int iters[yas::kMaxLevels] = {0};
    double K[9];
    cudaStream_t stream = nullptr;
    yas::LevelCam cam[yas::kMaxLevels];
    double dK[yas::kMaxLevels][4];  // double fx, fy, cx, cy per level
    yas::TrackLevelBufs set[2][yas::kMaxLevels];
    float *gx[yas::kMaxLevels] = {nullptr};
    float *gy[yas::kMaxLevels] = {nullptr};
    int cur = 0;  // current-frame set; the reference set is 1 - cur
    float4 *res4 = nullptr;       // per-pixel photometric residual (level-0 sized)
    float *partialA = nullptr;    // kMaxCtas x 32 per-CTA rows
    float *partialB = nullptr;    // kMaxCtas x 32
    float *growA = nullptr;       // per-group (hi, lo) rows of pass A
    float *growB = nullptr;       // per-group (hi, lo) rows of pass B
    unsigned *counters = nullptr; // tickets: pass A grid + groups, then pass B grid + groups
    unsigned long long *fused_rows = nullptr;  // fused schedule: tagged per-CTA rows
    bool use_fused = true;        // one cooperative launch for the whole schedule
    int fused_max_grid[4] = {-1, -1, -1, -1};  // co-resident CTAs for 1, 2, 4 pixels per thread, and any
    yas::GNState *state = nullptr;
    yas::GNState *state_host = nullptr;  // pinned
    void *staging = nullptr;             // host-input staging (w*h*4 bytes)
    size_t staging_bytes = 0;
    bool good = true;
    float angle_th, dist_th;      // ICP gates: sin(20 deg), 0.01 m
    std::vector<void *> allocations;
    // optional launch hook (profiling): called with a stage id before each pass
    void (*hook)(void *, int) = nullptr;
    void *hook_ctx = nullptr;

    yas::TrackLevelBufs &curb(int l) { return set[cur][l]; }
    yas::TrackLevelBufs &refb(int l) { return set[1 - cur][l]; }
};

namespace yas {
// Tracker passes (tracker.cu)
int tracker_alloc(yas_tracker *tr);
void tracker_free(yas_tracker *tr);
// Initialises the GN state with estimate `init` (host pose copied by value
// into a kernel argument, so it can be captured into a graph).
void launch_gn_init(yas_tracker *tr, const Pose64 &init, cudaStream_t s);
// One GN iteration at level l (pass A, and pass B for modes with RGB).
void launch_gn_iteration(yas_tracker *tr, int l, bool first_of_level, cudaStream_t s);
// Full coarse-to-fine schedule (GetTransform without the swap).
void launch_gn_schedule(yas_tracker *tr, cudaStream_t s);
// Preprocessing of current / reference frames from device sources.
void tracker_image(yas_tracker *tr, const uint8_t *src, int channels, int pitch, bool reference,
                   cudaStream_t s);
void tracker_depth(yas_tracker *tr, const void *src, int is_u16, int pitch, float scale, float *depth_m,
                   bool reference, cudaStream_t s);
void tracker_model(yas_tracker *tr, cudaStream_t s);  // model pyramid from ref vmap[0]
// Batched Gauss-Newton (many trackers, one cooperative launch):
// CTAs a tracker takes in a batch: one per `pixels_per_cta` level-0 pixels, 1..16
int gn_batch_ctas(const yas_tracker *tr, int pixels_per_cta = 32768);
// descriptor of its current frame
void gn_batch_item(yas_tracker *tr, int cta0, GNBatchItem *out, int pixels_per_cta = 32768);
// the same with an explicit CTA count (1..kFusedMaxCtas)
void gn_batch_item_ctas(yas_tracker *tr, int cta0, int nctas, GNBatchItem *out);
// the batched kernel's pixels-per-thread variant for these (host) descriptors:
// 1, 2, 4 (residuals in registers) or 0 (any share)
int gn_batch_pix(const GNBatchItem *items, int n);
int gn_batch_capacity();                                // co-resident CTAs of the batched launch
cudaError_t launch_gn_batch(const GNBatchItem *dev_items, const unsigned short *dev_cta_item, int grid,
                            cudaStream_t s, int pix);
}  // namespace yas
