/* Stand-in for the glm type named by the Camera declaration (include/Camera.h); the
 * camera code itself is not compiled. TEST INFRASTRUCTURE. */
#ifndef YREF_STUB_GLM_MAT4X4
#define YREF_STUB_GLM_MAT4X4
#include "vec4.hpp"
namespace glm {
struct mat4x4 {
  vec4 c[4];
};
typedef mat4x4 mat4;
}  // namespace glm
#endif
