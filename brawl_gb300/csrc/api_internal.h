// api_internal.h -- helpers the C-ABI translation units share (not exported
// through include/brawl_gpu.h).
#pragma once

#include <string>

#include "../../include/brawl_gpu.h"
#include "chain_engine.cuh"

namespace brawl {

// Records msg as the calling thread's last error and returns code.
int api_fail(int code, const std::string& msg);
// Validates a brawl_setup and derives the lattice geometry.
int api_make_geom(const brawl_setup& s, Geom& g);

}  // namespace brawl
