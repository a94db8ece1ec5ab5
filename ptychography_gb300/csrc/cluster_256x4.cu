// 256 x 256 frames on 4-CTA clusters (see cluster_frame.cuh).
#include "cluster_frame.cuh"

PTY_CLUSTER_TILE(256, 4)
