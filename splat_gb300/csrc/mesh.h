// mesh.h -- OBJ ingest into FTri records (host).
#pragma once

#include <string>
#include <vector>

#include "splat.h"

namespace splat {

// Parses a Wavefront OBJ file into FTri records, one per triangle of every
// face (polygons fan-triangulated).  Returns false with a message on error.
bool obj_to_ftri(const char* path, std::vector<splat_ftri_t>& out, std::string& err);

}  // namespace splat
