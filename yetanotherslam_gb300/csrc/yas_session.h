// yas_session.h — the parts of a session that the request server drives: one
// frame is copied in, then launched either as the initialising frame or as a
// tracked frame in two halves around the Gauss-Newton schedule (which the
// server runs for many sessions in one batched launch).
#pragma once

#include "yas_track.h"

struct yas_session;

namespace yas {

// Launch shapes of a session's kernels (chosen by the batch autotuner).  The
// march and integration shapes do not change any result; the GN share sets
// how a batched Gauss-Newton launch partitions the session's pixels, so it
// fixes the session's summation order.
struct LaunchShape {
    int march_warps_x = 2;       // ray march: 1, 2, 4 warp tiles across a CTA; 0 persistent (tile queue)
    int integrate_ctas = 0;      // integration grid (0: 152 x 8)
    int gn_pixels_per_cta = 32768;  // batched GN: one CTA per this many level-0 pixels
};

// Copies one frame (RGB u8 interleaved, depth u16) into the session's device
// buffers on its stream.
int session_copy_input(yas_session *s, const uint8_t *rgb, const uint16_t *depth, int on_device);
// True before the session's first frame (which initialises, without tracking).
bool session_needs_init(const yas_session *s);
// The initialising frame: reference pyramids and the first fusion.
int session_launch_first(yas_session *s);
// A tracked frame, first half: pyramids, raycast, model pyramid, GN reset.
// The Gauss-Newton schedule of the tracker's current frame sets follows.
int session_launch_pre(yas_session *s);
// A tracked frame, second half: pose update, fusion, frame state to the host;
// then swaps the tracker's frame sets.
int session_launch_post(yas_session *s);
yas_tracker *session_tracker(yas_session *s);
yas_map *session_map_handle(yas_session *s);
const yas_session_config &session_config(const yas_session *s);
// Launch shape; setting it drops the session's captured graphs.
void session_set_shape(yas_session *s, const LaunchShape &shape);
const LaunchShape &session_shape(const yas_session *s);
// Stream work of one frame without launching or bookkeeping, for a caller
// that captures many sessions into one graph (the batch): the initialising
// frame, or a tracked frame's halves around the Gauss-Newton schedule.
void session_enqueue_first(yas_session *s);
void session_enqueue_pre(yas_session *s);
void session_enqueue_post(yas_session *s);
// Bookkeeping after such a frame has been launched.
void session_finish_first(yas_session *s);
void session_finish_tracked(yas_session *s);
// Empties the map and restarts the session at its initialising frame.
int session_restart(yas_session *s);
cudaStream_t session_stream(yas_session *s);
// Pose and status of the last frame, once the session stream has completed it.
void session_result(const yas_session *s, yas_pose *Tcm, int *status);

}  // namespace yas
