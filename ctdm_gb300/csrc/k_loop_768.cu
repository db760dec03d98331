// Positivity-loop passes for 768^3 volumes, all plan variants (fft_line.cuh PV<768, v>).
#include "loop_passes.cuh"

CTDM_LOOP_SIZE_3(768)
