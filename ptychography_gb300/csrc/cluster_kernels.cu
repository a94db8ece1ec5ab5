// 256 x 256 frames: one frame per 4-CTA cluster (placeholder until the
// distributed-shared-memory transform lands).
#include "engine.h"

namespace pty {
bool cluster_frame_supported() { return false; }
int prepare_cluster_frame_kernels() { return set_error(PTY_ERR_SHAPE, "256x256 frames not built"); }
int launch_cluster_frame_op(int, const FrameArgs&, int, cudaStream_t) {
  return set_error(PTY_ERR_SHAPE, "256x256 frames not built");
}
}  // namespace pty
