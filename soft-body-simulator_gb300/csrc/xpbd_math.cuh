// Device math of the XPBD hot path: FP32 3x3 SVD and the per-constraint
// projections.  Every routine works on registers only; the kernels in
// xpbd_kernels.cu do the gathers and scatters.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sbs {

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 mk(float4 a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// 3x3 matrix as three columns.
struct m3 {
    f3 c0, c1, c2;
};

// F = Ds * DmInv with Ds = [d1 d2 d3] (columns) and DmInv given by its rows
// r0, r1, r2:  F = d1 r0^T + d2 r1^T + d3 r2^T.
__device__ __forceinline__ m3 deformation(f3 d1, f3 d2, f3 d3, f3 r0, f3 r1, f3 r2) {
    m3 F;
    F.c0 = d1 * r0.x + d2 * r1.x + d3 * r2.x;
    F.c1 = d1 * r0.y + d2 * r1.y + d3 * r2.y;
    F.c2 = d1 * r0.z + d2 * r1.z + d3 * r2.z;
    return F;
}

__device__ __forceinline__ float det3(const m3& F) { return dot(F.c0, cross(F.c1, F.c2)); }

// The Jacobi rotation in plane (p, q) is skipped when its off-diagonal is
// negligible.
template <int P, int Q>
__device__ __forceinline__ bool jacobi_skips(const float (&S)[3][3]) {
    return fabsf(S[P][Q]) <= 1e-30f + 1e-9f * (fabsf(S[P][P]) + fabsf(S[Q][Q]));
}

// One cyclic-Jacobi rotation on the symmetric matrix S (upper triangle
// s00 s01 s02 s11 s12 s22) in plane (p, q), accumulating into V's columns.
// Rotation from the symmetric 2x2 Schur decomposition (Golub & Van Loan,
// Matrix Computations, algorithm 8.4.1).  The rotation angle needs no IEEE
// division or square root: any (c, s) with c^2 + s^2 = 1 keeps V orthogonal
// and the sweeps converge the same, so tau and t use the fast reciprocal and
// sqrt(q) = q rsqrt(q) (14% off a frame of the 450-tet StVK beam).
template <int P, int Q>
__device__ __forceinline__ void jacobi_rot(float (&S)[3][3], f3 (&V)[3]) {
    const float spq = S[P][Q];
    const float spp = S[P][P], sqq = S[Q][Q];
    if (jacobi_skips<P, Q>(S)) return;
    const float tau = __fdividef(sqq - spp, 2.0f * spq);
    const float q = 1.0f + tau * tau;
    const float t = __fdividef(copysignf(1.0f, tau), fabsf(tau) + q * rsqrtf(q));
    const float c = rsqrtf(1.0f + t * t), s = t * c;
    constexpr int R = 3 - P - Q;
    S[P][P] = spp - t * spq;
    S[Q][Q] = sqq + t * spq;
    S[P][Q] = S[Q][P] = 0.0f;
    const float srp = S[R][P], srq = S[R][Q];
    S[R][P] = S[P][R] = c * srp - s * srq;
    S[R][Q] = S[Q][R] = s * srp + c * srq;
    const f3 vp = V[P], vq = V[Q];
    V[P] = vp * c - vq * s;
    V[Q] = vp * s + vq * c;
}

// SVD of F in the convention of Eigen's JacobiSVD: F = U diag(s) V^T with
// s >= 0 in decreasing order (U, V orthogonal, either handedness).
// Method: cyclic Jacobi eigen-decomposition of F^T F for V (at most 5
// sweeps), ordering by eigenvalue, then U from Gram-Schmidt on the columns of
// F V.  A tet's sweeps stop early once the next sweep would skip all three
// rotations (jacobi_rot's own test), when nothing would change any more: the
// result is bit-identical to five sweeps.  The test is the tet's own (not a
// warp vote), so it does not depend on which tets share a warp.
__device__ __forceinline__ void svd3(const m3& F, f3 (&U)[3], float (&s)[3], f3 (&V)[3]) {
    float S[3][3];
    S[0][0] = dot(F.c0, F.c0);
    S[1][1] = dot(F.c1, F.c1);
    S[2][2] = dot(F.c2, F.c2);
    S[0][1] = S[1][0] = dot(F.c0, F.c1);
    S[0][2] = S[2][0] = dot(F.c0, F.c2);
    S[1][2] = S[2][1] = dot(F.c1, F.c2);
    V[0] = mk(1.f, 0.f, 0.f);
    V[1] = mk(0.f, 1.f, 0.f);
    V[2] = mk(0.f, 0.f, 1.f);
#pragma unroll
    for (int sweep = 0; sweep < 5; ++sweep) {
        jacobi_rot<0, 1>(S, V);
        jacobi_rot<0, 2>(S, V);
        jacobi_rot<1, 2>(S, V);
        if (sweep < 4 && jacobi_skips<0, 1>(S) && jacobi_skips<0, 2>(S) && jacobi_skips<1, 2>(S)) break;
    }
    float e0 = S[0][0], e1 = S[1][1], e2 = S[2][2];
    // sort eigenvalues (and V columns) descending
    if (e0 < e1) { float t = e0; e0 = e1; e1 = t; f3 v = V[0]; V[0] = V[1]; V[1] = v; }
    if (e0 < e2) { float t = e0; e0 = e2; e2 = t; f3 v = V[0]; V[0] = V[2]; V[2] = v; }
    if (e1 < e2) { float t = e1; e1 = e2; e2 = t; f3 v = V[1]; V[1] = V[2]; V[2] = v; }
    // B = F V
    auto mulF = [&](f3 v) { return F.c0 * v.x + F.c1 * v.y + F.c2 * v.z; };
    f3 b0 = mulF(V[0]), b1 = mulF(V[1]), b2 = mulF(V[2]);
    const float q0 = dot(b0, b0);
    const float i0 = q0 > 1e-36f ? rsqrtf(q0) : 0.0f;
    float n0 = q0 * i0;
    f3 u0 = q0 > 1e-36f ? b0 * i0 : mk(1.f, 0.f, 0.f);
    f3 b1p = b1 - u0 * dot(u0, b1);
    const float q1 = dot(b1p, b1p);
    const float i1 = q1 > 1e-36f ? rsqrtf(q1) : 0.0f;
    float n1 = q1 * i1;
    f3 u1;
    if (n1 > 1e-7f * n0 && q1 > 1e-36f) {
        u1 = b1p * i1;
    } else {
        f3 e = fabsf(u0.x) < 0.9f ? mk(1.f, 0.f, 0.f) : mk(0.f, 1.f, 0.f);
        f3 wv = e - u0 * dot(e, u0);
        u1 = wv * rsqrtf(dot(wv, wv));
        n1 = fmaxf(n1, 0.0f);
    }
    f3 u2 = cross(u0, u1);
    float s2 = dot(u2, b2);
    if (s2 < 0.0f) { s2 = -s2; u2 = -u2; }
    U[0] = u0; U[1] = u1; U[2] = u2;
    s[0] = n0; s[1] = n1; s[2] = s2;
}

// Result of one tet evaluation: constraint value and the four gradients.
struct TetEval {
    float C;
    f3 g[4];
};

// Green-strain StVK energy constraint, following
// green_constraint_t::project_positions (src/physics/xpbd/green_constraint.cpp:61-120):
// inversion test by volume sign, SVD, sigma_3 flip when inverted, clamp at
// 0.577, Ehat, Phat, E = U Ehat V^T (as written there), psi, P = U Phat V^T,
// H = -|V0| P DmInv^T.  Returns C = |V0| psi and g_i = -f_i = grad_i C.
__device__ __forceinline__ void stvk_eval(f3 x0, f3 x1, f3 x2, f3 x3, f3 r0, f3 r1, f3 r2,
                                          float V0, float mu, float lam, TetEval& out) {
    const f3 d1 = x0 - x3, d2 = x1 - x3, d3 = x2 - x3;
    const float Vs = dot(d1, cross(d2, d3)) * (1.0f / 6.0f);
    const bool inverted = (Vs >= 0.0f) != (V0 >= 0.0f);
    const m3 F = deformation(d1, d2, d3, r0, r1, r2);
    f3 U[3], Vm[3];
    float s[3];
    svd3(F, U, s, Vm);
    if (inverted) { s[2] = -s[2]; U[2] = -U[2]; }
    const float min_sv = 0.577f;
    s[0] = fmaxf(s[0], min_sv);
    s[1] = fmaxf(s[1], min_sv);
    s[2] = fmaxf(s[2], min_sv);
    const float e0 = 0.5f * (s[0] * s[0] - 1.0f);
    const float e1 = 0.5f * (s[1] * s[1] - 1.0f);
    const float e2 = 0.5f * (s[2] * s[2] - 1.0f);
    const float etr = e0 + e1 + e2;
    const float p0 = s[0] * (2.0f * mu * e0 + lam * etr);
    const float p1 = s[1] * (2.0f * mu * e1 + lam * etr);
    const float p2 = s[2] * (2.0f * mu * e2 + lam * etr);
    // ||U Ehat V^T||_F^2 = sum e_i^2 ; tr(U Ehat V^T) = sum e_i (u_i . v_i)
    const float Etr = e0 * dot(U[0], Vm[0]) + e1 * dot(U[1], Vm[1]) + e2 * dot(U[2], Vm[2]);
    const float psi = mu * (e0 * e0 + e1 * e1 + e2 * e2) + 0.5f * lam * Etr * Etr;
    const float aV0 = fabsf(V0);
    out.C = aV0 * psi;
    // g_j = |V0| P r_j with P r = sum_i p_i u_i (v_i . r)
    auto Pr = [&](f3 r) {
        return U[0] * (p0 * dot(Vm[0], r)) + U[1] * (p1 * dot(Vm[1], r)) + U[2] * (p2 * dot(Vm[2], r));
    };
    out.g[0] = Pr(r0) * aV0;
    out.g[1] = Pr(r1) * aV0;
    out.g[2] = Pr(r2) * aV0;
    out.g[3] = -(out.g[0] + out.g[1] + out.g[2]);
}

// XPBD multiplier update of the StVK constraint (green_constraint.cpp:122-157).
// Returns dlambda (0 when the weighted gradient norm is below 1e-20); the
// quotient by the fast reciprocal, as it ends the per-tet latency chain.
__device__ __forceinline__ float stvk_dlambda(const TetEval& e, const float (&w)[4], float lam_acc,
                                              float alpha_tilde, float gamma, float gd) {
    const float S = w[0] * dot(e.g[0], e.g[0]) + w[1] * dot(e.g[1], e.g[1]) +
                    w[2] * dot(e.g[2], e.g[2]) + w[3] * dot(e.g[3], e.g[3]);
    if (S < 1e-20f) return 0.0f;
    const float num = -(e.C + alpha_tilde * lam_acc) + gamma * gd;
    const float den = (1.0f + gamma) * S + alpha_tilde;
    return __fdividef(num, den);
}

// Stable Neo-Hookean (Macklin & Mueller 2021), coupled 2x2 solve of the
// deviatoric C_D = ||F||_F (compliance 1/(mu|V0|)) and hydrostatic
// C_H = det F - (1 + mu/lam) (compliance 1/(lam|V0|)) constraints.
// Computes the position deltas dx[i] (already weighted by w_i) and the two
// multiplier increments.  Returns false when the step is skipped.  1/|F| by
// rsqrt and the other quotients by the fast reciprocal (a few ulp; the
// one-sweep parity against the FP64 oracle is unchanged at ~1e-6 of the
// scene diagonal): they sit on the per-phase latency chain, and the change
// took 9% off a frame of the 98k-tet beam.
__device__ __forceinline__ bool snh_step(f3 x0, f3 x1, f3 x2, f3 x3, f3 r0, f3 r1, f3 r2,
                                         float aV0, float mu, float lam, float inv_dt2,
                                         const float (&w)[4], float lamD, float lamH,
                                         f3 (&dx)[4], float& dlD, float& dlH) {
    const f3 d1 = x0 - x3, d2 = x1 - x3, d3 = x2 - x3;
    const m3 F = deformation(d1, d2, d3, r0, r1, r2);
    const float cD2 = dot(F.c0, F.c0) + dot(F.c1, F.c1) + dot(F.c2, F.c2);
    if (!(cD2 > 1e-24f)) return false;
    const float icD = rsqrtf(cD2);
    const float cD = cD2 * icD;
    const float J = det3(F);
    const float cH = J - (1.0f + __fdividef(mu, lam));
    const float atD = __fdividef(inv_dt2, mu * aV0), atH = __fdividef(inv_dt2, lam * aV0);
    // dC_D/dF = F / cD ; dC_H/dF = cof(F) = [f1 x f2 ... ] columns (f2 x f3, f3 x f1, f1 x f2)
    const f3 h0 = cross(F.c1, F.c2), h1 = cross(F.c2, F.c0), h2 = cross(F.c0, F.c1);
    // gradient wrt vertex j (j<3) = (dC/dF) r_j ; vertex 3 = -sum
    f3 gD[4], gH[4];
    gD[0] = (F.c0 * r0.x + F.c1 * r0.y + F.c2 * r0.z) * icD;
    gD[1] = (F.c0 * r1.x + F.c1 * r1.y + F.c2 * r1.z) * icD;
    gD[2] = (F.c0 * r2.x + F.c1 * r2.y + F.c2 * r2.z) * icD;
    gD[3] = -(gD[0] + gD[1] + gD[2]);
    gH[0] = h0 * r0.x + h1 * r0.y + h2 * r0.z;
    gH[1] = h0 * r1.x + h1 * r1.y + h2 * r1.z;
    gH[2] = h0 * r2.x + h1 * r2.y + h2 * r2.z;
    gH[3] = -(gH[0] + gH[1] + gH[2]);
    float a11 = atD, a22 = atH, a12 = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        a11 += w[i] * dot(gD[i], gD[i]);
        a22 += w[i] * dot(gH[i], gH[i]);
        a12 += w[i] * dot(gD[i], gH[i]);
    }
    const float b1 = -(cD + atD * lamD), b2 = -(cH + atH * lamH);
    const float det = a11 * a22 - a12 * a12;
    if (!(det > 1e-30f * a11 * a22)) return false;
    const float idet = __fdividef(1.0f, det);
    dlD = (b1 * a22 - b2 * a12) * idet;
    dlH = (b2 * a11 - b1 * a12) * idet;
#pragma unroll
    for (int i = 0; i < 4; ++i) dx[i] = (gD[i] * dlD + gH[i] * dlH) * w[i];
    return true;
}

// Residual terms of one SNH tet at the current positions.
// Compensated FP32 sum (Neumaier's variant of Kahan summation; pairs
// combined with Knuth's two-sum) for residuals and energies.
struct CSum {
    float s, e;
    __device__ __forceinline__ void add(float x) {
        const float t = s + x;
        if (fabsf(s) >= fabsf(x)) e += (s - t) + x;
        else e += (x - t) + s;
        s = t;
    }
    __device__ __forceinline__ void merge(const CSum& o) {
        add(o.s);
        e += o.e;
    }
};

__device__ __forceinline__ void snh_residual(f3 x0, f3 x1, f3 x2, f3 x3, f3 r0, f3 r1, f3 r2, float aV0,
                                             float mu, float lam, float inv_dt2, float lamD, float lamH,
                                             float& res2, float& energy) {
    const m3 F = deformation(x0 - x3, x1 - x3, x2 - x3, r0, r1, r2);
    const float cD2 = dot(F.c0, F.c0) + dot(F.c1, F.c1) + dot(F.c2, F.c2);
    const float cD = sqrtf(cD2);
    const float cH = det3(F) - (1.0f + mu / lam);
    const float hD = cD + inv_dt2 / (mu * aV0) * lamD;
    const float hH = cH + inv_dt2 / (lam * aV0) * lamH;
    res2 = hD * hD + hH * hH;
    energy = aV0 * (0.5f * mu * (cD2 - 3.0f) + 0.5f * lam * cH * cH);
}

}  // namespace sbs
