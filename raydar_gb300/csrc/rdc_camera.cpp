// rdc_camera.cpp -- Camera::update_matrices (src/scene/camera.rs:210-231)
// for the scene generator and for callers that edit a camera: view =
// look_at_lh(position, target, up), proj = GL-style perspective or ortho,
// and both inverses.  Host code only; compiled with -ffp-contract=off.
//
// Every entry is evaluated in float with the published formulas of cgmath
// 0.18.0 (the version the reference pins), in their order of operations, so
// the four matrices equal the reference's bit for bit (the tests pin them
// against the matrices stored in the reference's own scene files).
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

// 3x3 determinant of m (m[col][row]) expanded along its first row, as
// cgmath's Matrix3::determinant groups it:
// m00 (m11 m22 - m21 m12) - m10 (m01 m22 - m21 m02) + m20 (m01 m12 - m11 m02).
float det3(const float m[3][3]) {
    const float t0 = m[1][1] * m[2][2] - m[2][1] * m[1][2];
    const float t1 = m[0][1] * m[2][2] - m[2][1] * m[0][2];
    const float t2 = m[0][1] * m[1][2] - m[1][1] * m[0][2];
    return m[0][0] * t0 - m[1][0] * t1 + m[2][0] * t2;
}

// 3x3 matrix whose column k is row rows[k] of the column-major 4x4 `a`
// restricted to the columns cols[0..2] (a minor, laid out transposed).
void minor_by_rows(const float a[16], const int rows[3], const int cols[3], float m[3][3]) {
    for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) m[k][l] = a[cols[l] * 4 + rows[k]];
}

// The three indices of 0..3 other than `skip`, ascending.
void others(int skip, int out[3]) {
    for (int i = 0, n = 0; i < 4; ++i)
        if (i != skip) out[n++] = i;
}

// Inverse of a column-major 4x4 matrix by cofactors, as cgmath 0.18.0's
// Matrix4::invert computes it in float: det by expansion along row 0 with
// transposed minors of rows 1..3, singular when |det| <= f32::EPSILON (its
// ulps_eq! test against zero), then entry (column i, row j) =
// det3(minor without row i and column j, transposed) * (+-1) * (1 / det).
bool invert_cgmath(const float a[16], float out[16]) {
    static const int kRows123[3] = {1, 2, 3};
    float dk[4];
    for (int k = 0; k < 4; ++k) {
        int cols[3];
        others(k, cols);
        float m[3][3];
        minor_by_rows(a, kRows123, cols, m);
        dk[k] = det3(m);
    }
    const float det = a[0] * dk[0] - a[4] * dk[1] + a[8] * dk[2] - a[12] * dk[3];
    if (!(std::fabs(det) > 1.1920929e-7f)) return false;  // singular or NaN: the reference unwraps None
    const float inv_det = 1.0f / det;
    for (int i = 0; i < 4; ++i) {
        int rows[3];
        others(i, rows);
        for (int j = 0; j < 4; ++j) {
            int cols[3];
            others(j, cols);
            float m[3][3];
            minor_by_rows(a, rows, cols, m);
            const float sign = ((i + j) & 1) ? -1.0f : 1.0f;
            out[i * 4 + j] = det3(m) * sign * inv_det;
        }
    }
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
    if (!invert_cgmath(cam->view_matrix, cam->inverse_view_matrix)) return RDC_ERR_INVALID_ARGUMENT;
    if (!invert_cgmath(cam->proj_matrix, cam->inverse_proj_matrix)) return RDC_ERR_INVALID_ARGUMENT;
    return RDC_OK;
}
