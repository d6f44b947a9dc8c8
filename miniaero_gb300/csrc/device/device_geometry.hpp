// Device engine for the mesh geometry (geometry.cu).
#pragma once
#include <memory>
#include <string>

#include "../host/mesh.hpp"

namespace miniaero {

// A GeometryEngine that computes face and cell geometry on the current CUDA
// device, bit-identical to the host path; nullptr with *err set when the
// device cannot be used.
std::unique_ptr<GeometryEngine> make_device_geometry(std::string* err);

}  // namespace miniaero
