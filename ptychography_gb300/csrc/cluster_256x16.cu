// 256 x 256 frames on 16-CTA clusters of 128 threads (see cluster_frame.cuh).
#include "cluster_frame.cuh"

PTY_CLUSTER_TILE(256, 16)
