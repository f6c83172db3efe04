// svd3.cuh - 3x3 singular value decomposition for the particle return maps.
//
// Method (this project's own): cyclic Jacobi eigen-solve of the symmetric
// B = F^T F (the symmetric update of each rotation, which zeroes its pivot exactly),
// a descending sort of the eigenvalues,
// then a Givens QR of W = F V. U = Q and V are proper rotations; sigma = diag(R),
// so sigma_1 >= sigma_2 >= |sigma_3| and sigma_3 carries the sign of det F. That
// is the convention the material laws are written against (sigma_3 may be
// negative; the callers clamp with max()/abs()).
//
// Precision: the whole solve runs in FP32 registers. Coinciding singular values
// need no special branch: V may be any basis of the degenerate subspace and U
// follows from the QR of F V, so U diag(sigma) V^T still reproduces F. Only a
// near-singular F (sigma_3 < 1e-3 sigma_1), where F^T F in FP32 loses sigma_3,
// is redone in FP64.
#pragma once

namespace gbmpm {

template <typename T>
__device__ __forceinline__ T gb_sqrt(T x);
template <>
__device__ __forceinline__ float gb_sqrt<float>(float x) { return sqrtf(x); }
template <>
__device__ __forceinline__ double gb_sqrt<double>(double x) { return sqrt(x); }

template <typename T>
__device__ __forceinline__ T gb_rsqrt(T x);
template <>
__device__ __forceinline__ float gb_rsqrt<float>(float x) { return __frsqrt_rn(x); }   // correctly rounded
template <>
__device__ __forceinline__ double gb_rsqrt<double>(double x) { return 1.0 / sqrt(x); }

// One Jacobi rotation of the symmetric B in the (p, q) plane (r is the third index):
// the rotation that zeroes B[p][q] is applied to the diagonal, to the two entries of
// row r and, by symmetry, column r, and B[p][q] is set to zero (the classic
// symmetric update: B'pp = Bpp - t Bpq, B'qq = Bqq + t Bpq, B'rp = c Brp - s Brq,
// B'rq = s Brp + c Brq with t = sgn(theta) / (|theta| + sqrt(theta^2 + 1)),
// theta = (Bqq - Bpp) / (2 Bpq), c = 1 / sqrt(t^2 + 1), s = t c); V accumulates
// the rotation.
template <typename T>
__device__ __forceinline__ void jacobi_rot(T (&B)[3][3], T (&V)[3][3], int p, int q, int r) {
    const T bpq = B[p][q];
    if (bpq == T(0)) return;
    const T theta = (B[q][q] - B[p][p]) / (T(2) * bpq);
    const T at = theta < T(0) ? -theta : theta;
    T t;
    if (at > T(1e18)) t = T(0.5) / theta;
    else t = (theta >= T(0) ? T(1) : T(-1)) / (at + gb_sqrt<T>(theta * theta + T(1)));
    const T c = gb_rsqrt<T>(t * t + T(1));
    const T s = t * c;
    B[p][p] = B[p][p] - t * bpq;
    B[q][q] = B[q][q] + t * bpq;
    B[p][q] = T(0);
    B[q][p] = T(0);
    const T brp = B[r][p], brq = B[r][q];
    const T nrp = c * brp - s * brq, nrq = s * brp + c * brq;
    B[r][p] = nrp; B[p][r] = nrp;
    B[r][q] = nrq; B[q][r] = nrq;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T vkp = V[k][p], vkq = V[k][q];
        V[k][p] = c * vkp - s * vkq;
        V[k][q] = s * vkp + c * vkq;
    }
}

template <typename T>
__device__ __forceinline__ void swap_col(T (&V)[3][3], T (&B)[3][3], int a, int b) {
    T t = B[a][a]; B[a][a] = B[b][b]; B[b][b] = t;
#pragma unroll
    for (int k = 0; k < 3; ++k) { T u = V[k][a]; V[k][a] = V[k][b]; V[k][b] = -u; }
}

template <typename T>
__device__ __forceinline__ void givens_qr(T (&W)[3][3], T (&Q)[3][3], int a, int b, int col) {
    T x = W[a][col], y = W[b][col];
    T r = gb_sqrt<T>(x * x + y * y);
    T c = T(1), s = T(0);
    if (r > T(0)) { c = x / r; s = y / r; }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T wa = W[a][k], wb = W[b][k];
        W[a][k] = c * wa + s * wb;
        W[b][k] = -s * wa + c * wb;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T qa = Q[k][a], qb = Q[k][b];
        Q[k][a] = c * qa + s * qb;
        Q[k][b] = -s * qa + c * qb;
    }
}

// F row-major in, U and V row-major rotations out, s descending (s[2] signed).
template <typename T>
__device__ __forceinline__ void svd3_t(const float* F, float* U, float* s, float* Vout) {
    T A[3][3], B[3][3], V[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) A[i][j] = (T)F[3 * i + j];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            B[i][j] = A[0][i] * A[0][j] + A[1][i] * A[1][j] + A[2][i] * A[2][j];
            V[i][j] = (i == j) ? T(1) : T(0);
        }
    const T tol = sizeof(T) == 4 ? T(1e-14) : T(1e-30);
    for (int sweep = 0; sweep < (sizeof(T) == 4 ? 8 : 20); ++sweep) {
        T off = B[0][1] * B[0][1] + B[0][2] * B[0][2] + B[1][2] * B[1][2];
        T dia = B[0][0] * B[0][0] + B[1][1] * B[1][1] + B[2][2] * B[2][2];
        if (off <= tol * dia) break;
        jacobi_rot<T>(B, V, 0, 1, 2);
        jacobi_rot<T>(B, V, 0, 2, 1);
        jacobi_rot<T>(B, V, 1, 2, 0);
    }
    // descending sort; each swap negates one column so V stays proper
    if (B[0][0] < B[1][1]) swap_col<T>(V, B, 0, 1);
    if (B[0][0] < B[2][2]) swap_col<T>(V, B, 0, 2);
    if (B[1][1] < B[2][2]) swap_col<T>(V, B, 1, 2);
    T W[3][3], Q[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            W[i][j] = A[i][0] * V[0][j] + A[i][1] * V[1][j] + A[i][2] * V[2][j];
            Q[i][j] = (i == j) ? T(1) : T(0);
        }
    givens_qr<T>(W, Q, 0, 1, 0);
    givens_qr<T>(W, Q, 0, 2, 0);
    givens_qr<T>(W, Q, 1, 2, 1);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) { U[3 * i + j] = (float)Q[i][j]; Vout[3 * i + j] = (float)V[i][j]; }
    s[0] = (float)W[0][0];
    s[1] = (float)W[1][1];
    s[2] = (float)W[2][2];
}

__device__ __forceinline__ void svd3(const float* F, float* U, float* s, float* V) {
    svd3_t<float>(F, U, s, V);
    float a2 = fabsf(s[2]);
    if (!(a2 >= 1e-3f * s[0])) svd3_t<double>(F, U, s, V);
}

}  // namespace gbmpm
