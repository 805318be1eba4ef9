// yas_session.h — the parts of a session that the request server drives: one
// frame is copied in, then launched either as the initialising frame or as a
// tracked frame in two halves around the Gauss-Newton schedule (which the
// server runs for many sessions in one batched launch).
#pragma once

#include "yas_track.h"

struct yas_session;

namespace yas {

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
cudaStream_t session_stream(yas_session *s);
// Pose and status of the last frame, once the session stream has completed it.
void session_result(const yas_session *s, yas_pose *Tcm, int *status);

}  // namespace yas
