// Oracle (test infrastructure only): camera matrices of Lumen's PerspectiveCamera.
//
// Follows src/Framework/Camera.h:67-74 (view = lookAtLH(pos, pos + dir, up (0,1,0))), Camera.h:109-116
// (projection with the Vulkan y flip) and src/RayTracer/Integrator.cpp:67-68 (the shader receives the
// inverses). glm is not vendored, so lookAtLH and the 4x4 inverse are written from their textbook
// definitions; the inverse is formed in double precision and rounded once to FP32.
// Camera.h:75-84 also round-trips the view through a quaternion and XYZ Euler angles; for a camera
// looking along +z that round trip is the identity, which is how every procedural scene here is set up.
#include <cmath>

#include "oracle.h"

namespace {
void invert4(const double m[16], double out[16]) {
    // Cofactor expansion on a column-major matrix m[4*c + r].
    double inv[16];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    for (int i = 0; i < 16; i++) out[i] = inv[i] / det;
}
}  // namespace

extern "C" void orc_camera_matrices(const float pos[3], const float dir[3], float fov_deg, uint32_t width,
                                    uint32_t height, float inv_view[16], float inv_proj[16]) {
    // projection (Camera.h:109-116), column-major proj[4*c + r]
    const float cam_near = 0.01f, cam_far = 1000.0f;
    const float aspect = (float)width / (float)height;
    const float half = fov_deg / 2.0f * (3.14159265358979323846f / 180.0f);
    double P[16] = {0};
    for (int i = 0; i < 4; i++) P[5 * i] = 1.0;
    P[0] = 1.0f / (aspect * std::tan(half));
    P[5] = -1.0f / std::tan(half);
    P[10] = cam_far / (cam_near - cam_far);
    P[11] = -1.0;  // [2][3]
    P[14] = cam_near * cam_far / (cam_near - cam_far);  // [3][2]
    P[15] = 1.0;  // glm::mat4{1.f} starts as identity; [3][3] is never overwritten
    // lookAtLH(eye, center = eye + dir, up)
    double eye[3] = {pos[0], pos[1], pos[2]};
    double f[3] = {dir[0], dir[1], dir[2]};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& x : f) x /= fl;
    double up[3] = {0, 1, 0};
    double s[3] = {up[1] * f[2] - up[2] * f[1], up[2] * f[0] - up[0] * f[2], up[0] * f[1] - up[1] * f[0]};
    double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    for (double& x : s) x /= sl;
    double u[3] = {f[1] * s[2] - f[2] * s[1], f[2] * s[0] - f[0] * s[2], f[0] * s[1] - f[1] * s[0]};
    double V[16] = {0};
    V[15] = 1.0;
    V[0] = s[0]; V[4] = s[1]; V[8] = s[2];
    V[1] = u[0]; V[5] = u[1]; V[9] = u[2];
    V[2] = f[0]; V[6] = f[1]; V[10] = f[2];
    V[12] = -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2]);
    V[13] = -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]);
    V[14] = -(f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2]);
    double iv[16], ip[16];
    invert4(V, iv);
    invert4(P, ip);
    for (int i = 0; i < 16; i++) { inv_view[i] = (float)iv[i]; inv_proj[i] = (float)ip[i]; }
}
