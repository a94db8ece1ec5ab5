// 512 x 512 frames on 16-CTA clusters (see cluster_frame.cuh).
#include "cluster_frame.cuh"

PTY_CLUSTER_TILE(512, 16)
