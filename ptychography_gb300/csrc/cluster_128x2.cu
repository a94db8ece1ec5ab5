// 128 x 128 frames on 2-CTA clusters (see cluster_frame.cuh).
#include "cluster_frame.cuh"

PTY_CLUSTER_TILE(128, 2)
