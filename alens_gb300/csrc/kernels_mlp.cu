// kernels_mlp.cu - learned warm start (placeholder translation unit).
#include "engine.cuh"
