/*
 * dio_selftest.h -- entry points that run the device-wide primitives of the
 * pipeline on host arrays, for tests that compare them with host results.
 * They are not part of the drop-in boundary (dio_cuda.h): no reference
 * interface corresponds to them.
 *
 * Each call allocates its device buffers, runs on a private stream, copies
 * the result back and frees everything before it returns.  Status codes are
 * those of dio_cuda.h (DIO_ERR_TIMEOUT when a bounded look-back wait gave up).
 */
#ifndef DIO_SELFTEST_H
#define DIO_SELFTEST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* out[i] = in[0] + ... + in[i-1] (uint32 wrap-around) for i < min(live, n),
 * with `live` handed to the kernel in device memory as the pipeline's
 * device counts are; out[i] for larger i is left as it was.  *total (may be
 * null) receives the sum of the live entries.  Computed `repeats` times in a
 * row (>= 1) on the same buffers. */
int dio_selftest_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t live, uint32_t repeats,
                      uint32_t* total);

/* Stable sort of (keys[i], vals[i]) by key bits [begin_bit, end_bit); the
 * other key bits ride along.  end_bit <= 32 (u32) or 64 (u64). */
int dio_selftest_sort_u32(const uint32_t* keys, const uint32_t* vals, uint32_t n, uint32_t begin_bit,
                          uint32_t end_bit, uint32_t* keys_out, uint32_t* vals_out);
int dio_selftest_sort_u64(const uint64_t* keys, const uint32_t* vals, uint32_t n, uint32_t begin_bit,
                          uint32_t end_bit, uint64_t* keys_out, uint32_t* vals_out);

#ifdef __cplusplus
}
#endif
#endif
