// Stand-in for the CUDA samples' helper_functions.h (timers and string parsing the
// reference's headers include but the comparison build does not use).
#pragma once
