// Mirrors the reference header of the same path (parthenon-hpc-lab/parthenon src/globals.hpp):
// the compatibility layer declares everything in one place.
#pragma once
#include "pgb_compat/all.hpp"
