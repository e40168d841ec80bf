// A small vector/matrix library with the names, storage and conventions of
// the glm calls that the reference's CUDA sources make (src/fluid.cu,
// src/virt.cu, src/solid.cu, src/pair.cu, include/*.cuh).  glm itself is not
// vendored by the reference and is absent here, so these types and functions
// are written from their mathematical definitions:
//
//   vec3   three floats x, y, z (12 bytes, no padding), v[i] indexes them;
//   mat3   three column vectors (36 bytes, column-major): m[c][r] is the
//          entry in column c, row r; mat3(s) is s times the identity;
//   A * B  the matrix product, column c of A*B = A * (column c of B);
//   M * v  the matrix-vector product, sum over c of column c times v[c];
//   outerProduct(c, r) = c r^T, column j = c * r[j];
//   determinant  cofactor expansion along the first column;
//   inverse      adjugate (transposed cofactors) times 1/determinant;
//   normalize(v) = v * (1 / sqrt(dot(v, v)));  length(v) = sqrt(dot(v, v)).
//
// Test infrastructure only: it lets the reference's unmodified device code be
// compiled into the reference build that the GPU parity tests and the
// reference bench arm load.  Roundings may differ from the real glm's in the
// last bit; the parity tests compare within stated tolerances.
#ifndef FSIM_REF_GLM_SUBSET_HPP
#define FSIM_REF_GLM_SUBSET_HPP

#include <math.h>

#if defined(__CUDACC__)
#define FSIM_GLM_FN __host__ __device__ inline
#else
#define FSIM_GLM_FN inline
#endif

namespace glm {

struct vec3 {
    float x, y, z;
    FSIM_GLM_FN vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    FSIM_GLM_FN explicit vec3(float s) : x(s), y(s), z(s) {}
    FSIM_GLM_FN vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    FSIM_GLM_FN float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    FSIM_GLM_FN const float &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    FSIM_GLM_FN vec3 &operator+=(const vec3 &o) { x += o.x; y += o.y; z += o.z; return *this; }
    FSIM_GLM_FN vec3 &operator-=(const vec3 &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    FSIM_GLM_FN vec3 &operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    FSIM_GLM_FN vec3 &operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};

FSIM_GLM_FN vec3 operator+(const vec3 &a, const vec3 &b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
FSIM_GLM_FN vec3 operator-(const vec3 &a, const vec3 &b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
FSIM_GLM_FN vec3 operator-(const vec3 &a) { return vec3(-a.x, -a.y, -a.z); }
FSIM_GLM_FN vec3 operator*(const vec3 &a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
FSIM_GLM_FN vec3 operator*(float s, const vec3 &a) { return vec3(s * a.x, s * a.y, s * a.z); }
FSIM_GLM_FN vec3 operator*(const vec3 &a, const vec3 &b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
FSIM_GLM_FN vec3 operator/(const vec3 &a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

// Equality is exact and component-wise (so a NaN component makes v == v false).
FSIM_GLM_FN bool operator==(const vec3 &a, const vec3 &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
FSIM_GLM_FN bool operator!=(const vec3 &a, const vec3 &b) { return !(a == b); }

FSIM_GLM_FN float dot(const vec3 &a, const vec3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
FSIM_GLM_FN float length(const vec3 &a) { return sqrtf(dot(a, a)); }
FSIM_GLM_FN vec3 normalize(const vec3 &a) { return a * (1.0f / sqrtf(dot(a, a))); }

struct mat3 {
    vec3 col[3];
    FSIM_GLM_FN mat3() { col[0] = vec3(1.0f, 0.0f, 0.0f); col[1] = vec3(0.0f, 1.0f, 0.0f); col[2] = vec3(0.0f, 0.0f, 1.0f); }
    FSIM_GLM_FN explicit mat3(float s) { col[0] = vec3(s, 0.0f, 0.0f); col[1] = vec3(0.0f, s, 0.0f); col[2] = vec3(0.0f, 0.0f, s); }
    FSIM_GLM_FN mat3(const vec3 &c0, const vec3 &c1, const vec3 &c2) { col[0] = c0; col[1] = c1; col[2] = c2; }
    FSIM_GLM_FN vec3 &operator[](int i) { return col[i]; }
    FSIM_GLM_FN const vec3 &operator[](int i) const { return col[i]; }
    FSIM_GLM_FN mat3 &operator+=(const mat3 &o) { col[0] += o.col[0]; col[1] += o.col[1]; col[2] += o.col[2]; return *this; }
    FSIM_GLM_FN mat3 &operator-=(const mat3 &o) { col[0] -= o.col[0]; col[1] -= o.col[1]; col[2] -= o.col[2]; return *this; }
};

FSIM_GLM_FN mat3 operator+(const mat3 &a, const mat3 &b) { return mat3(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
FSIM_GLM_FN mat3 operator-(const mat3 &a, const mat3 &b) { return mat3(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
FSIM_GLM_FN mat3 operator*(const mat3 &a, float s) { return mat3(a[0] * s, a[1] * s, a[2] * s); }
FSIM_GLM_FN mat3 operator*(float s, const mat3 &a) { return mat3(s * a[0], s * a[1], s * a[2]); }
FSIM_GLM_FN mat3 operator/(const mat3 &a, float s) { return mat3(a[0] / s, a[1] / s, a[2] / s); }
FSIM_GLM_FN vec3 operator*(const mat3 &m, const vec3 &v) { return m[0] * v.x + m[1] * v.y + m[2] * v.z; }
FSIM_GLM_FN mat3 operator*(const mat3 &a, const mat3 &b) { return mat3(a * b[0], a * b[1], a * b[2]); }

FSIM_GLM_FN mat3 transpose(const mat3 &m)
{
    return mat3(vec3(m[0].x, m[1].x, m[2].x), vec3(m[0].y, m[1].y, m[2].y), vec3(m[0].z, m[1].z, m[2].z));
}

FSIM_GLM_FN mat3 outerProduct(const vec3 &c, const vec3 &r) { return mat3(c * r.x, c * r.y, c * r.z); }

// Cofactor C(r, c) of entry (row r, column c) of m, m(r, c) = m[c][r].
FSIM_GLM_FN float glm_subset_minor(const mat3 &m, int r0, int r1, int c0, int c1)
{
    return m[c0][r0] * m[c1][r1] - m[c1][r0] * m[c0][r1];
}

FSIM_GLM_FN float determinant(const mat3 &m)
{
    // expansion along column 0: sum over rows r of m(r, 0) * C(r, 0)
    return m[0][0] * glm_subset_minor(m, 1, 2, 1, 2) - m[0][1] * glm_subset_minor(m, 0, 2, 1, 2) +
           m[0][2] * glm_subset_minor(m, 0, 1, 1, 2);
}

FSIM_GLM_FN mat3 inverse(const mat3 &m)
{
    // inverse(r, c) = C(c, r) / det; C(c, r) = (-1)^(r+c) * minor without row c, column r
    float c00 = glm_subset_minor(m, 1, 2, 1, 2), c10 = -glm_subset_minor(m, 0, 2, 1, 2), c20 = glm_subset_minor(m, 0, 1, 1, 2);
    float c01 = -glm_subset_minor(m, 1, 2, 0, 2), c11 = glm_subset_minor(m, 0, 2, 0, 2), c21 = -glm_subset_minor(m, 0, 1, 0, 2);
    float c02 = glm_subset_minor(m, 1, 2, 0, 1), c12 = -glm_subset_minor(m, 0, 2, 0, 1), c22 = glm_subset_minor(m, 0, 1, 0, 1);
    float det = m[0][0] * c00 + m[0][1] * c10 + m[0][2] * c20;
    float inv = 1.0f / det;
    // column c of the inverse holds the cofactors of row c of m: (C(c,0), C(c,1), C(c,2))
    return mat3(vec3(c00 * inv, c01 * inv, c02 * inv), vec3(c10 * inv, c11 * inv, c12 * inv),
                vec3(c20 * inv, c21 * inv, c22 * inv));
}

}  // namespace glm

#endif
