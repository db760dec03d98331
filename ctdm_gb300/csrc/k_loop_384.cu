// Positivity-loop passes for 384^3 volumes, all plan variants (fft_line.cuh PV<384, v>).
#include "loop_passes.cuh"

CTDM_LOOP_SIZE_3(384)
