// Shared declarations between the host driver (iris_host.cpp) and the CUDA
// engine (iris_engine.cu, iris_batch.cu, iris_adjoint.cu).  Not part of the
// public ABI.
#pragma once
#include <string>

#include "iris_fdtd.h"

namespace iris {

// Record a message for iris_last_error() and return code.
int fail(int code, const std::string& msg);
void clear_error();

// Engine-side helpers used by the host driver.
long engine_npts(const iris_engine* eng, int box, int j);

}  // namespace iris
