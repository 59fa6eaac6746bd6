// Float-float evaluation of one table cell in difference form (FfRec),
// shared by the mixed-precision lookups of the tabulated models
// (sgx_lookup_mixed.cu, sgx_lookup_sie.cu).
#pragma once

#include "sgx_ff.cuh"
#include "sgx_spiner.cuh"

namespace sgx {

// The record's field f = x + a dT + b dR + a b dRT at (a, b); AB = a b.
// The three products and the four-term sum leave their low parts
// unnormalised; ff2d takes the sum as it is.
__device__ __forceinline__ ff ff_cell(const FfRec &r, const ff A, const ff B, const ff AB) {
  const ff x = ff_make(r.x[0], r.x[1]);
  const ff t = ff_mul_nn(A, ff_make(r.dT[0], r.dT[1]));
  const ff d = ff_mul_nn(B, ff_make(r.dR[0], r.dR[1]));
  const ff c = ff_mul_nn(AB, ff_make(r.dRT[0], r.dRT[1]));
  return ff_sum4(x, t, d, c);
}

// One 32-byte record per lane in one 256-bit load (records are 32-byte
// aligned): a random gather then costs one instruction per record.
__device__ __forceinline__ FfRec load_rec(const FfRec *p) {
  FfRec r;
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(r.x[0]), "=f"(r.x[1]), "=f"(r.dT[0]), "=f"(r.dT[1]), "=f"(r.dR[0]), "=f"(r.dR[1]),
        "=f"(r.dRT[0]), "=f"(r.dRT[1])
      : "l"(p));
  return r;
}
} // namespace sgx
