// Butcher tables by ARKODE table number (butcher.cu).
#pragma once

#include "common.cuh"

namespace gbmv {

constexpr int kMaxStages = GBMV_MAX_STAGES;

struct ButcherTable {
  int id;
  const char* name;
  int s;  // stages
  int q;  // order of the method
  int p;  // order of the embedding
  double c[kMaxStages];
  double A[kMaxStages][kMaxStages];  // row i: a_i0 .. a_ii (diagonal included)
  double b[kMaxStages];
  double bhat[kMaxStages];
};

// The table with this number, or null.
const ButcherTable* butcher_table(int id);
// ARKODE's default explicit table of an order (2-5), or -1.
int erk_default_table(int order);

}  // namespace gbmv
