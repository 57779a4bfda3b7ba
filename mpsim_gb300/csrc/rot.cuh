// Jacobi rotation parameters shared by the FP32 SIMT sweep kernel
// (jacobi.cu) and the tensor-core block sweep (tcjacobi.cu).
#pragma once

#include "common.cuh"

namespace mps {

// Squared cosine of the angle between two columns, |gamma|^2 / (a b).  A pair
// rotates when it exceeds tol^2, and the per-job maximum of the same value
// decides convergence, so a sweep that rotates nothing always ends the job.
// Zero columns give 0; when g2 = |gamma|^2 or a norm is below the smallest
// normal float, the cosine is formed from |gamma| and the square roots of the
// norms with IEEE operations instead.
__device__ __forceinline__ float pair_cos2(cf gam, float g2, float a, float b) {
    const float kMinNormal = 1.17549435e-38f;
    if (g2 >= kMinNormal && a >= kMinNormal && b >= kMinNormal)
        return __fdividef(__fdividef(g2, a), b);
    // |gamma|^2 underflows once the columns are below ~1e-10 in norm (graded
    // columns, as the L factor has from the start): take |gamma| itself.
    // Pairs with a + b below 1e-36 leave no room for the rotation's
    // 1/(a+b) and count as orthogonal.
    if (!(a > 0.f && b > 0.f) || !(a + b >= 1e-36f)) return 0.f;
    const float r = (hypotf(gam.x, gam.y) / sqrtf(a)) / sqrtf(b);
    return r * r;
}

// The rotation of a pair in the form
//   x <- x - (tp x + sigma q),   q <- q + (conj(sigma) x - tp q),
// sigma = s conj(gamma)/|gamma|, tp = 1 - c = s^2 / (1 + c): the complex
// Jacobi rotation [[c, -sigma], [conj(sigma), c]], with c kept implicit as
// 1 - tp (see the file comment).  It equals the rotation with the unit phase
// e = conj(gamma)/|gamma| applied to q (q <- e q + ...) followed by conj(e)
// on the new q, which changes no norm and no orthogonality.  dn = t |gamma|
// is the norm transfer: |x'|^2 = a - dn, |q'|^2 = b + dn.
struct Rot {
    float tp, dn;
    cf sigma;
};

// Rotation parameters for gamma != 0 from quantities scaled by u = 1/(a+b)
// (gamma u is squared, not gamma: no overflow or underflow for a + b >= 1e-36):
// t = sign(b-a) 2|gamma| / (|b-a| + sqrt((b-a)^2 + 4|gamma|^2)),
// c = 1/sqrt(1+t^2) (approximate reciprocal square root refined by one
// Newton step), s = c t.  |sigma|^2 and tp come from the same c^2 t^2, so
// rounding perturbs a rotated column's norm by a few ulps times s^2 only.
__device__ __forceinline__ Rot make_rot(float a, float b, cf gam) {
    const float ab = a + b;
    const float u = ab >= 1e-30f ? __fdividef(1.f, ab) : 1.f / ab;
    const float p = b - a;
    const float ph = p * u;                              // in [-1, 1]
    const float gx = gam.x * u, gy = gam.y * u;
    const float gh = fmaf(gx, gx, gy * gy);              // |gamma|^2 u^2, in (0, 1/4]
    const float h = fmaf(ph, ph, 4.f * gh);
    const float th = __fdividef(2.f, fabsf(ph) + h * rsqrtf(h));   // |t| / (|gamma| u)
    const float t2 = gh * th * th;                       // t^2 <= 1
    const float x = 1.f + t2;
    float c = rsqrtf(x);
    c = c * fmaf(-0.5f * x * c, c, 1.5f);                // Newton step for 1/sqrt(x)
    const float sg = p >= 0.f ? 1.f : -1.f;
    const float k = c * sg * u * th;                     // sigma = k conj(gamma)
    Rot r;
    r.sigma = cmake(k * gam.x, -k * gam.y);
    r.tp = __fdividef(c * c * t2, 1.f + c);
    r.dn = sg * gh * th * ab;                            // = sg |gamma|^2 u th
    return r;
}

__device__ __forceinline__ void apply_rot(const Rot& r, cf& x, cf& q) {
    const float sr = r.sigma.x, si = r.sigma.y, tp = r.tp;
    float nxr = fmaf(-tp, x.x, x.x), nxi = fmaf(-tp, x.y, x.y);
    float nqr = fmaf(-tp, q.x, q.x), nqi = fmaf(-tp, q.y, q.y);
    nxr = fmaf(-sr, q.x, nxr);
    nxi = fmaf(-sr, q.y, nxi);
    nqr = fmaf(sr, x.x, nqr);
    nqi = fmaf(sr, x.y, nqi);
    nxr = fmaf(si, q.y, nxr);
    nxi = fmaf(-si, q.x, nxi);
    nqr = fmaf(si, x.y, nqr);
    nqi = fmaf(-si, x.x, nqi);
    x = cmake(nxr, nxi);
    q = cmake(nqr, nqi);
}

}  // namespace mps
