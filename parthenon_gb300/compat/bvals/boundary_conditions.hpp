// Mirrors the reference header of the same path (parthenon-hpc-lab/parthenon src/bvals/boundary_conditions.hpp):
// the compatibility layer declares everything in one place.
#pragma once
#include "../pgb_compat/all.hpp"
