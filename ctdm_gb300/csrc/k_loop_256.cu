// Positivity-loop passes for 256^3 volumes, all plan variants (fft_line.cuh PV<256, v>).
#include "loop_passes.cuh"

CTDM_LOOP_SIZE_3(256)
