// Conversion of the C ABI's flat pg_feature_params into pg::FeatureParams.
#pragma once

#include "model_tables.h"
#include "polymlp_gb300.h"

namespace pg {

// Validates shapes and ranges; throws std::runtime_error on bad input.
FeatureParams feature_params_from_abi(const pg_feature_params* p);

}  // namespace pg
