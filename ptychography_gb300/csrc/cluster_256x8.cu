// 256 x 256 frames on 8-CTA clusters (see cluster_frame.cuh).
#include "cluster_frame.cuh"

PTY_CLUSTER_TILE(256, 8)
