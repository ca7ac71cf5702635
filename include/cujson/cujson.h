// cujson.h -- drop-in for the reference's standard-JSON umbrella header
// (cujson/cujson.h): loaders, parse_standard_json and cuJSONIterator, backed by
// libcujson_gb300.  Link with -lcujson_gb300 (and the CUDA runtime).
#pragma once
#include "cujson_types.h"
#include "cujson_api.h"
#include "cujson_iter.h"
