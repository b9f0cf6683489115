// hyc_tmap.h -- host-side TMA descriptors (CUtensorMap) of FP64 and FP32
// slice arrays, shared by the plain-form and ensemble host layers.
#pragma once
#include <cuda.h>

#include <cstdint>

namespace hyc {

// cuTensorMapEncodeTiled is reachable through the runtime's driver
// entry-point query
bool tmap_available();

// 3-D tiled map over nz slices of w x h elements (row pitch ld1, slice pitch
// sl, both in elements; element size es = 4 or 8), box bx x by x 1, zero
// fill outside.  False when the driver refuses it or when the TMA rules do
// not hold: base 16-byte aligned, row and slice pitches multiples of 16
// bytes, box rows a multiple of 16 bytes.
bool tmap_encode3(CUtensorMap *m, const void *base, int es, long long w, long long h, long long ld1, long long sl,
                  long long nz, int bx, int by);

}  // namespace hyc
