// yh_camera.cpp -- Cam buffer of Yune's Camera, restated without glm.
//
// Camera::setViewMatrix (src/Camera.cpp:105-117) normalises side/up/look and builds
// the view-to-world matrix with columns (side, up, -look, eye); Camera::setBuffer
// (src/Camera.cpp:66-82) writes its rows r1..r4 into Cam. view_plane_dist is
// 1/tan(yFOV*3.14/360), evaluated in double as the reference does (the literal 3.14,
// not pi; src/Camera.cpp:49,62).
#include "yune_host.h"

#include <cmath>

namespace {
// glm::normalize(vec4): v * inversesqrt(dot(v, v)); glm's vec4 dot sums
// (x*x + y*y) + (z*z + w*w).
void normalize4(const float in[4], float out[4]) {
  const float d = (in[0] * in[0] + in[1] * in[1]) + (in[2] * in[2] + in[3] * in[3]);
  const float inv = 1.0f / std::sqrt(d);
  for (int i = 0; i < 4; ++i) out[i] = in[i] * inv;
}
}  // namespace

extern "C" int yh_camera_look(const float eye[3], const float side[3], const float up[3],
                              const float look[3], float y_fov_deg, yc_cam* out) {
  if (!eye || !side || !up || !look || !out) return YH_E_INVALID;
  const float s4[4] = {side[0], side[1], side[2], 0.0f};
  const float u4[4] = {up[0], up[1], up[2], 0.0f};
  const float l4[4] = {look[0], look[1], look[2], 0.0f};
  float s[4], u[4], l[4];
  normalize4(s4, s);
  normalize4(u4, u);
  normalize4(l4, l);
  // columns: side, up, -look, eye ; rows are read across the columns
  const float col[4][4] = {{s[0], s[1], s[2], s[3]},
                           {u[0], u[1], u[2], u[3]},
                           {-l[0], -l[1], -l[2], -l[3]},
                           {eye[0], eye[1], eye[2], 1.0f}};
  yc_float4* rows[4] = {&out->r1, &out->r2, &out->r3, &out->r4};
  for (int r = 0; r < 4; ++r) *rows[r] = yc_float4{col[0][r], col[1][r], col[2][r], col[3][r]};
  out->view_plane_dist = (float)(1 / std::tan((double)y_fov_deg * 3.14 / 360));
  out->pad[0] = out->pad[1] = out->pad[2] = 0.0f;
  return YH_OK;
}
