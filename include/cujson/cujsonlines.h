// cujsonlines.h -- drop-in for the reference's JSON-Lines umbrella header
// (cujson/cujsonlines.h): loaders, parse_json_lines and cuJSONLinesIterator,
// backed by libcujson_gb300.  Link with -lcujson_gb300 (and the CUDA runtime).
#pragma once
#include "cujson_types.h"
#include "cujson_api.h"
#include "cujson_iter.h"
