// Positivity-loop passes for 512^3 volumes, all plan variants (fft_line.cuh PV<512, v>).
#include "loop_passes.cuh"

CTDM_LOOP_SIZE_3(512)
