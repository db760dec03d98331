// Positivity-loop passes for the small volume sides 32, 64 and 128 (one plan each).
#include "loop_passes.cuh"

CTDM_LOOP_SIZE_1(32)
CTDM_LOOP_SIZE_1(64)
CTDM_LOOP_SIZE_1(128)
