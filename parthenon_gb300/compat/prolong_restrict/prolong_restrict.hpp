// Mirrors the reference header of the same path (parthenon-hpc-lab/parthenon src/prolong_restrict/prolong_restrict.hpp):
// the compatibility layer declares everything in one place.
#pragma once
#include "../pgb_compat/all.hpp"
