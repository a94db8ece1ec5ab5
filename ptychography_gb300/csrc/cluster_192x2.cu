// 192 x 192 frames on 2-CTA clusters (see cluster_frame.cuh).
#include "cluster_frame.cuh"

PTY_CLUSTER_TILE(192, 2)
