// Stand-in for nvpro_core's nvmath header (an empty submodule of the
// reference): the reference's src/shared/ headers include it in C++ mode to
// name their vector types.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "../../glsl_shim.h"
namespace nvmath {
using vec2f = glslx::vec2;
using vec3f = glslx::vec3;
using vec4f = glslx::vec4;
using mat4f = glslx::mat4;
using mat3f = glslx::mat3;
}  // namespace nvmath
