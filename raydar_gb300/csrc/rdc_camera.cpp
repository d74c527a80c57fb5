// rdc_camera.cpp -- Camera::update_matrices (src/scene/camera.rs:210-231)
// for the scene generator and for callers that edit a camera: view =
// look_at_lh(position, target, up), proj = GL-style perspective or ortho,
// and both inverses.  Host code only; compiled with -ffp-contract=off.
//
// The view and projection entries are evaluated in float with cgmath 0.18's
// published formulas.  The inverses are computed in double by Gauss-Jordan
// elimination with partial pivoting and rounded once to float; the
// reference's own float inversion differs from that by at most a few ulp
// (the tests pin both against the matrices stored in the reference scenes).
#include <cmath>
#include <cstring>

#include "raydar_cuda.h"

namespace {

struct F3 {
    float x, y, z;
};

F3 f3sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
float f3dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
F3 f3norm(F3 a) {
    const float inv = 1.0f / std::sqrt(f3dot(a, a));
    return {a.x * inv, a.y * inv, a.z * inv};
}
F3 f3cross(F3 a, F3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Inverse of a column-major 4x4 matrix; false if singular.
bool invert_gauss_jordan(const float in[16], float out[16]) {
    double m[4][8];
    for (int r = 0; r < 4; ++r) {
        for (int c = 0; c < 4; ++c) m[r][c] = in[c * 4 + r];
        for (int c = 0; c < 4; ++c) m[r][4 + c] = (r == c) ? 1.0 : 0.0;
    }
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (std::fabs(m[r][col]) > std::fabs(m[piv][col])) piv = r;
        if (m[piv][col] == 0.0 || !std::isfinite(m[piv][col])) return false;
        if (piv != col)
            for (int c = 0; c < 8; ++c) std::swap(m[piv][c], m[col][c]);
        const double p = m[col][col];
        for (int c = 0; c < 8; ++c) m[col][c] /= p;
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            const double f = m[r][col];
            if (f == 0.0) continue;
            for (int c = 0; c < 8; ++c) m[r][c] -= f * m[col][c];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = (float)m[r][4 + c];
    return true;
}

}  // namespace

extern "C" rdc_status rdc_camera_update_matrices(rdc_camera* cam) {
    if (!cam) return RDC_ERR_INVALID_ARGUMENT;
    if (cam->resolution_y == 0 || cam->resolution_x == 0) return RDC_ERR_INVALID_ARGUMENT;
    const F3 eye{cam->position[0], cam->position[1], cam->position[2]};
    const F3 tgt{cam->target[0], cam->target[1], cam->target[2]};
    const F3 up{cam->up[0], cam->up[1], cam->up[2]};

    // cgmath Matrix4::look_at_lh: f = normalize(target - eye),
    // s = normalize(up x f), u = f x s; rows s, u, f; translation -eye.(s,u,f).
    const F3 f = f3norm(f3sub(tgt, eye));
    const F3 s = f3norm(f3cross(up, f));
    const F3 u = f3cross(f, s);
    float* v = cam->view_matrix;
    const float view[16] = {s.x, u.x, f.x, 0.0f, s.y, u.y, f.y, 0.0f,
                            s.z, u.z, f.z, 0.0f, -f3dot(eye, s), -f3dot(eye, u), -f3dot(eye, f), 1.0f};
    std::memcpy(v, view, sizeof(view));

    const float aspect = (float)cam->resolution_x / (float)cam->resolution_y;
    const float near = cam->near_clip, far = cam->far_clip;
    float* p = cam->proj_matrix;
    for (int i = 0; i < 16; ++i) p[i] = 0.0f;
    if (cam->projection == RDC_PROJECTION_PERSPECTIVE) {
        // cgmath::perspective: f = cot(fovy/2) with fovy in radians.
        const float half = (cam->fov_degrees * (float)(3.14159265358979323846 / 180.0)) / 2.0f;
        const float fc = 1.0f / std::tan(half);
        p[0] = fc / aspect;
        p[5] = fc;
        p[10] = (far + near) / (near - far);
        p[11] = -1.0f;
        p[14] = (2.0f * far * near) / (near - far);
    } else if (cam->projection == RDC_PROJECTION_ORTHOGRAPHIC) {
        // cgmath::ortho(-size*aspect, size*aspect, -size, size, near, far).
        const float l = -cam->ortho_size * aspect, r = cam->ortho_size * aspect;
        const float b = -cam->ortho_size, t = cam->ortho_size;
        p[0] = 2.0f / (r - l);
        p[5] = 2.0f / (t - b);
        p[10] = -2.0f / (far - near);
        p[12] = -(r + l) / (r - l);
        p[13] = -(t + b) / (t - b);
        p[14] = -(far + near) / (far - near);
        p[15] = 1.0f;
    } else {
        return RDC_ERR_INVALID_ARGUMENT;
    }
    // The reference unwraps the inverses (camera.rs:229-230); a singular
    // matrix is reported here instead of panicking.
    if (!invert_gauss_jordan(cam->view_matrix, cam->inverse_view_matrix)) return RDC_ERR_INVALID_ARGUMENT;
    if (!invert_gauss_jordan(cam->proj_matrix, cam->inverse_proj_matrix)) return RDC_ERR_INVALID_ARGUMENT;
    return RDC_OK;
}
