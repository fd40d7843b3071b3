/* Stand-in for the glm type named by the Camera declaration (include/Camera.h); the
 * camera code itself is not compiled. TEST INFRASTRUCTURE. */
#ifndef YREF_STUB_GLM_VEC4
#define YREF_STUB_GLM_VEC4
namespace glm {
struct vec4 {
  float x, y, z, w;
};
}  // namespace glm
#endif
