// (q, dtype) -> (lattice, scalar type) dispatch for the C entry points.
#pragma once

#include "vs_common.cuh"

namespace vs {

template <typename T>
struct Tag {
  using type = T;
};

template <class F>
int dispatch(int q, int dtype, F&& fn) {
  if (dtype != VS_F32 && dtype != VS_F64) {
    set_error("dtype must be VS_F32 or VS_F64, got %d", dtype);
    return VS_ERR_INVALID_ARG;
  }
  if (q == 9) return dtype == VS_F32 ? fn(L9{}, Tag<float>{}) : fn(L9{}, Tag<double>{});
  if (q == 19) return dtype == VS_F32 ? fn(L19{}, Tag<float>{}) : fn(L19{}, Tag<double>{});
  set_error("q must be 9 (D2Q9) or 19 (D3Q19), got %d", q);
  return VS_ERR_INVALID_ARG;
}

template <class F>
int dispatch_t(int dtype, F&& fn) {
  if (dtype == VS_F32) return fn(Tag<float>{});
  if (dtype == VS_F64) return fn(Tag<double>{});
  set_error("dtype must be VS_F32 or VS_F64, got %d", dtype);
  return VS_ERR_INVALID_ARG;
}

}  // namespace vs
