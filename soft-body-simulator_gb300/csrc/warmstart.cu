// Learned warm start of a substep's Gauss-Seidel sweeps.
//
// After the prediction (timestep.cpp:35-43) the displacement the substep's
// solve will apply is guessed per vertex as d_i = d_prev_i + MLP(features_i):
// the solve displacement of the previous substep (the motion is smooth, so it
// is already close) plus a learned correction.  Moving the positions alone
// would break XPBD's bookkeeping (x - x_pred must stay sum_j M^-1 grad C_j^T
// lambda_j, with lambda starting at 0), so the guess is turned into
// multipliers by "fit" sweeps in the solver's colour order: each constraint
// takes the multiplier increment whose position update best matches the
// displacement still missing at its vertices,
//     dl = argmin sum_i m_i |w_i grad_i C dl - r_i|^2 + alpha~ (lambda + dl)^2,
//     r_i = x_pred_i + d_i - x_i,
// (2x2 normal equations for SNH), and moves its vertices accordingly.  The
// ordinary sweeps then continue from those multipliers.  With no fit sweeps
// the start "carries" the previous substep's multipliers instead (k_carry).
// Features (per
// vertex): x_pred - x (3), d_prev (3), Green strain of the mean deformation
// gradient of the incident tets at x_pred (6: E00 E11 E22 E01 E02 E12),
// external acceleration (3), pin flag (1).
#include <cuda_runtime.h>
#include <stdint.h>

#include "warmstart_internal.cuh"
#include "launch_count.cuh"
#include "xpbd_internal.cuh"
#include "xpbd_math.cuh"

namespace sbs {

// dprev_valid: w.xpred holds the prediction of the substep that produced the
// current x (features ran on it and the state was not replaced since), so
// x - w.xpred is that substep's solve displacement.
// Deformation gradient of every tet at the predicted positions, row-major in
// three float4 (each tet once, instead of once per incident vertex).
__global__ void k_tet_f(SceneDev s, WarmDev w) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < s.n_tets; t += gridDim.x * blockDim.x) {
        const uint4 id = s.tet[t];
        const f3 x3 = mk(s.xi[id.w]);
        const f3 d1 = mk(s.xi[id.x]) - x3, d2 = mk(s.xi[id.y]) - x3, d3 = mk(s.xi[id.z]) - x3;
        const m3 Fm = deformation(d1, d2, d3, mk(s.dm0[t]), mk(s.dm1[t]), mk(s.dm2[t]));
        w.tet_f[3ull * t] = make_float4(Fm.c0.x, Fm.c1.x, Fm.c2.x, 0.0f);
        w.tet_f[3ull * t + 1] = make_float4(Fm.c0.y, Fm.c1.y, Fm.c2.y, 0.0f);
        w.tet_f[3ull * t + 2] = make_float4(Fm.c0.z, Fm.c1.z, Fm.c2.z, 0.0f);
    }
}

// Eight lanes per vertex: each adds the gradients of every eighth incident
// tet in incidence order, the eight partial sums are added by a fixed
// shuffle tree, and the group's first lane writes the vertex's features (the
// loads of a vertex's ~24 incident tets are in flight together).
constexpr uint32_t kFeatLanes = 8;

__global__ void k_features(SceneDev s, WarmDev w, StepParams p, int dprev_valid) {
    const uint32_t sub = threadIdx.x & (kFeatLanes - 1);
    const uint32_t stride = gridDim.x * blockDim.x / kFeatLanes;
    // uniform trip count across the warp: every lane takes part in the shuffles
    const uint32_t n_pad = (s.n_verts + stride - 1) / stride * stride;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) / kFeatLanes; v < n_pad; v += stride) {
        const bool live = v < s.n_verts;
        float F[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const uint32_t b = live ? w.inc_start[v] : 0u, e = live ? w.inc_start[v + 1] : 0u;
        for (uint32_t k = b + sub; k < e; k += kFeatLanes) {
            const uint32_t t = w.inc[k];
            const float4 r0 = w.tet_f[3ull * t], r1 = w.tet_f[3ull * t + 1], r2 = w.tet_f[3ull * t + 2];
            F[0] += r0.x; F[1] += r0.y; F[2] += r0.z;
            F[3] += r1.x; F[4] += r1.y; F[5] += r1.z;
            F[6] += r2.x; F[7] += r2.y; F[8] += r2.z;
        }
#pragma unroll
        for (uint32_t o = kFeatLanes / 2; o > 0; o >>= 1)
#pragma unroll
            for (int i = 0; i < 9; ++i) F[i] += __shfl_xor_sync(0xffffffffu, F[i], o);
        if (!live || sub != 0) continue;
        const float4 xp = s.xi[v], x = s.xn[v];
        float f[16];
        f[0] = xp.x - x.x;
        f[1] = xp.y - x.y;
        f[2] = xp.z - x.z;
        if (dprev_valid) {
            const float4 xo = w.xpred[v];
            f[3] = x.x - xo.x;
            f[4] = x.y - xo.y;
            f[5] = x.z - xo.z;
        } else {
            f[3] = f[4] = f[5] = 0.0f;
        }
        // mean of the incident tets' gradients (k_tet_f)
        const float inv = e > b ? 1.0f / (float)(e - b) : 0.0f;
        for (int i = 0; i < 9; ++i) F[i] *= inv;
        // E = (F^T F - I) / 2 of the mean gradient (F row-major)
        const f3 c0 = mk(F[0], F[3], F[6]), c1 = mk(F[1], F[4], F[7]), c2 = mk(F[2], F[5], F[8]);
        f[6] = 0.5f * (dot(c0, c0) - 1.0f);
        f[7] = 0.5f * (dot(c1, c1) - 1.0f);
        f[8] = 0.5f * (dot(c2, c2) - 1.0f);
        f[9] = 0.5f * dot(c0, c1);
        f[10] = 0.5f * dot(c0, c2);
        f[11] = 0.5f * dot(c1, c2);
        const bool pinned = !(xp.w > 0.0f);
        float ax = 0.f, ay = 0.f, az = 0.f;
        if (!pinned) {
            if (p.gravity_mode == 1) { ax = p.gx * xp.w; ay = p.gy * xp.w; az = p.gz * xp.w; }
            else { ax = p.gx; ay = p.gy; az = p.gz; }
            if (p.has_acc && s.v[v].w == 0.0f) {
                const float4 a = s.acc[v];
                ax += a.x; ay += a.y; az += a.z;
            }
        }
        f[12] = ax;
        f[13] = ay;
        f[14] = az;
        f[15] = pinned ? 1.0f : 0.0f;
        // the row's 64 bytes as four 16-byte stores
        float4* out = reinterpret_cast<float4*>(w.feat + (size_t)v * 16);
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
        w.xpred[v] = xp;
    }
}

// One tet of a fit sweep; the first fit sweep of the substep starts the
// multipliers from 0, later ones accumulate.
__device__ __forceinline__ void fit_tet(const SceneDev& s, const WarmDev& w, const StepParams& p, uint32_t t,
                                        bool first) {
    const uint4 id = s.tet[t];
    const float4 a = s.dm0[t], b = s.dm1[t], c = s.dm2[t];
    float4 q[4] = {__ldcg(&s.xi[id.x]), __ldcg(&s.xi[id.y]), __ldcg(&s.xi[id.z]), __ldcg(&s.xi[id.w])};
    const uint32_t vid[4] = {id.x, id.y, id.z, id.w};
    f3 r[4];
    float wgt[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float4 xp = w.xpred[vid[i]];
        const float* d = w.delta + (size_t)vid[i] * 3;
        const float* dp = w.feat + (size_t)vid[i] * 16 + 3;
        r[i] = mk(xp.x + dp[0] + d[0] - q[i].x, xp.y + dp[1] + d[1] - q[i].y, xp.z + dp[2] + d[2] - q[i].z);
        wgt[i] = q[i].w;
    }
    const f3 x0 = mk(q[0]), x1 = mk(q[1]), x2 = mk(q[2]), x3 = mk(q[3]);
    const f3 r0 = mk(a), r1 = mk(b), r2 = mk(c);
    f3 dx[4];
    if (s.model[t] == 0) {
        TetEval e;
        stvk_eval(x0, x1, x2, x3, r0, r1, r2, a.w, b.w, c.w, e);
        float num = 0.f, den = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            num += wgt[i] > 0.0f ? dot(e.g[i], r[i]) : 0.0f;
            den += wgt[i] * dot(e.g[i], e.g[i]);
        }
        const float l0 = first ? 0.0f : s.lam0[t];
        const float dl = den > 1e-20f ? (num - p.stvk_alpha_tilde * l0) / (den + p.stvk_alpha_tilde) : 0.0f;
        s.lam0[t] = l0 + dl;
#pragma unroll
        for (int i = 0; i < 4; ++i) dx[i] = e.g[i] * (wgt[i] * dl);
    } else {
        const float aV0 = fabsf(a.w), mu = b.w, lam = c.w;
        const m3 F = deformation(x0 - x3, x1 - x3, x2 - x3, r0, r1, r2);
        const float cD = sqrtf(dot(F.c0, F.c0) + dot(F.c1, F.c1) + dot(F.c2, F.c2));
        const float lD = first ? 0.0f : s.lam0[t], lH = first ? 0.0f : s.lam1[t];
        float dlD = 0.f, dlH = 0.f;
        f3 gD[4], gH[4];
        if (cD > 1e-12f) {
            const float icD = 1.0f / cD;
            const f3 h0 = cross(F.c1, F.c2), h1 = cross(F.c2, F.c0), h2 = cross(F.c0, F.c1);
            gD[0] = (F.c0 * r0.x + F.c1 * r0.y + F.c2 * r0.z) * icD;
            gD[1] = (F.c0 * r1.x + F.c1 * r1.y + F.c2 * r1.z) * icD;
            gD[2] = (F.c0 * r2.x + F.c1 * r2.y + F.c2 * r2.z) * icD;
            gD[3] = -(gD[0] + gD[1] + gD[2]);
            gH[0] = h0 * r0.x + h1 * r0.y + h2 * r0.z;
            gH[1] = h0 * r1.x + h1 * r1.y + h2 * r1.z;
            gH[2] = h0 * r2.x + h1 * r2.y + h2 * r2.z;
            gH[3] = -(gH[0] + gH[1] + gH[2]);
            const float atD = p.inv_dt2 / (mu * aV0), atH = p.inv_dt2 / (lam * aV0);
            float a11 = atD, a22 = atH, a12 = 0.f, b1 = -atD * lD, b2 = -atH * lH;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a11 += wgt[i] * dot(gD[i], gD[i]);
                a22 += wgt[i] * dot(gH[i], gH[i]);
                a12 += wgt[i] * dot(gD[i], gH[i]);
                if (wgt[i] > 0.0f) {
                    b1 += dot(gD[i], r[i]);
                    b2 += dot(gH[i], r[i]);
                }
            }
            const float det = a11 * a22 - a12 * a12;
            if (det > 1e-30f * a11 * a22) {
                dlD = (b1 * a22 - b2 * a12) / det;
                dlH = (b2 * a11 - b1 * a12) / det;
            }
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) gD[i] = gH[i] = mk(0.f, 0.f, 0.f);
        }
        s.lam0[t] = lD + dlD;
        s.lam1[t] = lH + dlH;
#pragma unroll
        for (int i = 0; i < 4; ++i) dx[i] = (gD[i] * dlD + gH[i] * dlH) * wgt[i];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        q[i].x += dx[i].x;
        q[i].y += dx[i].y;
        q[i].z += dx[i].z;
        s.xi[vid[i]] = q[i];
    }
}

__global__ void k_fit_segment(SceneDev s, WarmDev w, StepParams p, uint32_t b, uint32_t e, int first) {
    for (uint32_t t = b + blockIdx.x * blockDim.x + threadIdx.x; t < e; t += gridDim.x * blockDim.x)
        fit_tet(s, w, p, t, first != 0);
}

// Carry start (no fit sweeps): every free vertex moves to x_pred + d_prev +
// MLP correction, and the multipliers keep the values the previous substep's
// solve ended with - the displacement d_prev came from those multipliers, so
// the two stay consistent up to the change of the constraint gradients over
// one substep.  For stiff bodies, whose Gauss-Seidel sweeps rebuild the
// multipliers only slowly, that start is far closer to the solution than
// multipliers fitted from the displacement in a few sweeps.
__global__ void k_carry(SceneDev s, WarmDev w) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n_verts; i += gridDim.x * blockDim.x) {
        float4 x = s.xi[i];
        if (!(x.w > 0.0f)) continue;
        const float* dp = w.feat + (size_t)i * 16 + 3;
        const float* d = w.delta + (size_t)i * 3;
        x.x += dp[0] + d[0];
        x.y += dp[1] + d[1];
        x.z += dp[2] + d[2];
        s.xi[i] = x;
    }
}

// Fallback of a judged substep whose warm start was discarded
// (JudgeDev::fallback, decided on the device): the positions go back to the
// prediction and the elastic multipliers to zero, i.e. the plain start.
__global__ void k_judge_fallback(SceneDev s, WarmDev w, const JudgeDev* j) {
    if (!j->fallback) return;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n_verts; i += stride) s.xi[i] = w.xpred[i];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < s.n_tets; t += stride) {
        s.lam0[t] = 0.0f;
        s.lam1[t] = 0.0f;
    }
}

// Totals of a judged substep once its sweep loop ended.
__global__ void k_judge_end(JudgeDev* j, int substep) {
    const double target = j->target[substep];
    j->warm_substeps++;
    j->total_sweeps += j->sweeps;
    if (!(j->r_now <= target)) j->capped++;
    const double ratio = target > 0.0 ? j->r_now / target : (j->r_now > 0.0 ? 1e30 : 1.0);
    j->sum_ratio += ratio;
    if (ratio > j->max_ratio) j->max_ratio = ratio;
}

cudaError_t launch_judge_fallback(const SceneDev& s, const WarmDev& w, const JudgeDev* j, cudaStream_t st) {
    const uint32_t n = s.n_verts > s.n_tets ? s.n_verts : s.n_tets;
    const int grid = (int)std::min<uint32_t>(2048, (n + 255) / 256);
    k_judge_fallback<<<grid > 0 ? grid : 1, 256, 0, st>>>(s, w, j);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_judge_end(JudgeDev* j, int substep, cudaStream_t st) {
    k_judge_end<<<1, 1, 0, st>>>(j, substep);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_carry(const SceneDev& s, const WarmDev& w, cudaStream_t st) {
    const int grid = (int)std::min<uint32_t>(4096, (s.n_verts + 255) / 256);
    k_carry<<<grid > 0 ? grid : 1, 256, 0, st>>>(s, w);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_features(const SceneDev& s, const WarmDev& w, const StepParams& p, int dprev_valid,
                            cudaStream_t st) {
    const int tgrid = (int)std::min<uint32_t>(4096, (s.n_tets + 255) / 256);
    k_tet_f<<<tgrid > 0 ? tgrid : 1, 256, 0, st>>>(s, w);
    count_launch();
    const int grid = (int)std::min<uint64_t>(4096, ((uint64_t)s.n_verts * kFeatLanes + 255) / 256);
    k_features<<<grid > 0 ? grid : 1, 256, 0, st>>>(s, w, p, dprev_valid);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_fit_segment(const SceneDev& s, const WarmDev& w, const StepParams& p, uint32_t b, uint32_t e,
                               int first, cudaStream_t st) {
    if (e <= b) return cudaSuccess;
    const int grid = (int)std::min<uint32_t>(2048, (e - b + 127) / 128);
    k_fit_segment<<<grid, 128, 0, st>>>(s, w, p, b, e, first);
    count_launch();
    return cudaGetLastError();
}

}  // namespace sbs
