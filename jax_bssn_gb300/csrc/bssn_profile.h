// Launch accounting: every kernel launch of the library goes through
// BSSN_LAUNCH, which counts it and, when profiling is enabled, brackets it
// with CUDA events on its own stream so per-kernel device time can be read
// back (bssn_profile_read).  Profiling is off by default.
#pragma once

#include <cuda_runtime.h>

namespace bssn {

enum KernelClass {
    KC_FILL = 0, KC_FIRST, KC_GAUGE, KC_KGT, KC_AT, KC_MOM_DERIVED, KC_MOM_DAMP, KC_SOMMERFELD,
    KC_STAGE, KC_PROJECT, KC_IMPORT, KC_EXPORT, KC_CONSTRAINTS, KC_TRANSFER, KC_CARTOON, KC_CONVERT, KC_OTHER,
    KC_CURV, KC_SOLVE_NEWTON, KC_SOLVE_APPLY, KC_SOLVE_UPDATE, KC_HORIZON_SURFACE, KC_HORIZON_SOLVE,
    KC_ADJ_POINT, KC_ADJ_STENCIL, KC_ADJ_STAGE,
    KC_COUNT
};

void prof_begin(int cls, cudaStream_t s);
// Per-launch event timing is on (bssn_profile_enable).
bool profiling_enabled();
// Adds n (may be negative) to the launch counter: kernels replayed from a
// CUDA graph, or recorded during a capture without running.
void count_launches(long long n);
void prof_end(int cls, cudaStream_t s);

}  // namespace bssn

#define BSSN_LAUNCH(cls, kernel, grid, block, stream, ...)          \
    do {                                                            \
        ::bssn::prof_begin((cls), (stream));                        \
        kernel<<<(grid), (block), 0, (stream)>>>(__VA_ARGS__);      \
        ::bssn::prof_end((cls), (stream));                          \
    } while (0)
