/*
 * The case descriptor as the XLA FFI handlers receive it: the bytes of a
 * gbf_case (include/gbfluids.h) as an int64 attribute "desc", packed on the
 * Python side by jaxfluids_gb300.jax_binding.pack_case (sizeof(gbf_case) is a
 * multiple of 8: the struct holds doubles and pointers).  Shared by the
 * handlers (gbf_ffi.cc) and by the test that checks the packing through the
 * C ABI without jaxlib.
 */
#ifndef GBF_FFI_DESC_H
#define GBF_FFI_DESC_H

#include <stdint.h>
#include <string.h>

#include "gbfluids.h"

#define GBF_DESC_WORDS (sizeof(gbf_case) / sizeof(int64_t))

/* Unpack `words` (n int64 words) into *out: GBF_OK, or
 * GBF_ERR_INVALID_ARGUMENT for a null pointer or a word count that is not
 * GBF_DESC_WORDS (a descriptor of another ABI version). */
static inline int gbf_case_from_words(const int64_t* words, size_t n, gbf_case* out) {
  if (!words || !out || n != GBF_DESC_WORDS) return GBF_ERR_INVALID_ARGUMENT;
  memcpy(out, words, sizeof(gbf_case));
  return GBF_OK;
}

#endif /* GBF_FFI_DESC_H */
