// Internal declarations shared by the C ABI translation units.
#pragma once

#include "mechanics.cuh"

namespace goal {

void states_to_host(Mechanics& m, int which, double* out);
void states_from_host(Mechanics& m, int which, const double* in);
void bsr_to_csr(const SolInfo& s, double* out_host);

}  // namespace goal
