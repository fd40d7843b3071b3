/* Stand-in for the glm vector type Yune's scene loader uses (src/Scene.cpp:247-330).
 * TEST INFRASTRUCTURE: lets Scene::loadModel compile for the oracle without glm. */
#ifndef YREF_STUB_GLM_VEC3
#define YREF_STUB_GLM_VEC3
namespace glm {
struct vec3 {
  float x, y, z;
};
}  // namespace glm
#endif
