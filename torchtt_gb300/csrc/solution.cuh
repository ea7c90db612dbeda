// The library-owned result handle behind the opaque ttgb_solution of include/ttgb300.h.
#pragma once

#include "amen.cuh"

struct ttgb_solution {
  ttgb::AmenResult res;
};

struct ttgb_amen_params;
namespace ttgb {
// Validated copy of the C parameter block (throws kInvalidArgument on bad values).
AmenParams params_from_c(const ttgb_amen_params* params);
}  // namespace ttgb
