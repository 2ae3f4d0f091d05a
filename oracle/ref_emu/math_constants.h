// Host stand-ins for the two constants of CUDA's math_constants.h that the reference's LBVH uses.
// Part of the host emulation in oracle/ref_emu (test infrastructure only).
#pragma once
#define CUDART_INF_F __builtin_huge_valf()
#define CUDART_INF __builtin_huge_val()
