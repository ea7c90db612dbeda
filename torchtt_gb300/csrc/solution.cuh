// The library-owned result handle behind the opaque ttgb_solution of include/ttgb300.h.
#pragma once

#include "amen.cuh"

struct ttgb_solution {
  ttgb::AmenResult res;
};
