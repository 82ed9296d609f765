#pragma once

// One complex float32 sample as stored in a .cf32 file: I then Q (src/types.hpp:7-12). An array
// of cf32 is the interleaved [I0, Q0, I1, Q1, ...] buffer the C ABI takes.
struct cf32 {
    float re;
    float im;
};

static_assert(sizeof(cf32) == 2 * sizeof(float), "cf32 must be two packed floats");
