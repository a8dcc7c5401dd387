// kz_device.cuh — device-side math, RNG, shading frame, Fresnel, microfacet
// distributions and closure lobes of the kazen hot path (sm_103a).
//
// Everything here computes in FP32 (a few reference expressions promote to
// double exactly where the reference does). The library is compiled with
// --fmad=false so every expression rounds as written.
//
// Reference formulas (paths within kazen_proto):
//   Frame / cos_theta / reflect / refract / fresnel .. src/base/utils.h:83-210
//   Fresnel (dielectric, Schlick) .................... src/shading/fresnel.h:12-187
//   GGX / Beckmann D, Lambda, G, G1, VNDF pdf ........ src/shading/microfacet.h:60-291
//   Diffuse, KpMirror, KpDielectric, KpGloss, KpGlass,
//   KpPrincipleSpecularReflection .................... src/shading/bsdfs.cpp:27-41,
//                                                      254-298, 359-554, 688-730
//   KpGlass reflection/refraction helpers ............ src/shading/bsdfs.h:541-599
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/kazen_gb300.h"

namespace kz {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kRayEps = 1e-4f;  // epsilon<float>, src/base/basic_types.h:9

struct f3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ f3 mk(float a, float b, float c) { return f3{a, b, c}; }
__host__ __device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__host__ __device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ f3 hmul(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__host__ __device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ __forceinline__ f3 normalize(f3 a) {
    float l = sqrtf(dot(a, a));
    return {a.x / l, a.y / l, a.z / l};
}
// base::Vec::normalized() of the reference (src/base/vec.h:784-790): the
// reciprocal length is taken in double and rounded once to float
__host__ __device__ __forceinline__ f3 normalize_ref(f3 a) {
    const float rcp = (float)(1.0 / sqrt((double)dot(a, a)));
    return {a.x * rcp, a.y * rcp, a.z * rcp};
}
template <bool kRefNorm>
__host__ __device__ __forceinline__ f3 nrm(f3 a) {
    return kRefNorm ? normalize_ref(a) : normalize(a);
}
__host__ __device__ __forceinline__ float sq(float a) { return a * a; }
__host__ __device__ __forceinline__ bool is_zero(f3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
__host__ __device__ __forceinline__ float max_comp(f3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__host__ __device__ __forceinline__ float comp(f3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// ------------------------------------------------------------------ PCG32
// PCG-XSH-RR 64/32 (M. O'Neill, "PCG: A Family of Simple Fast Space-Efficient
// Statistically Good Algorithms for Random Number Generation", 2014).
constexpr uint64_t kPcgMult = 6364136223846793005ULL;

__device__ __forceinline__ uint32_t pcg_output(uint64_t old) {
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return __funnelshift_r(xs, xs, rot);
}
struct Pcg {
    uint64_t state, inc;
    __device__ __forceinline__ void seed(uint64_t initstate, uint64_t initseq) {
        inc = (initseq << 1u) | 1u;
        state = 0u;
        state = state * kPcgMult + inc;
        state += initstate;
        state = state * kPcgMult + inc;
    }
    __device__ __forceinline__ uint32_t next() {
        uint64_t old = state;
        state = old * kPcgMult + inc;
        return pcg_output(old);
    }
    // 23 random mantissa bits in [1, 2) minus 1 (pcg32::nextFloat, the
    // generator behind the reference Sampler, src/core/sampler.cpp:22-27).
    __device__ __forceinline__ float nextf() { return __uint_as_float((next() >> 9) | 0x3f800000u) - 1.0f; }
};

// ------------------------------------------------------------------ frame
// Frame(n): normal -> local y, t chosen from the larger of |n.x|, |n.y|
// (src/base/utils.h:191-201).
struct Frame {
    f3 s, t, n;
    __device__ __forceinline__ explicit Frame(f3 nn) : n(nn) {
        if (fabsf(n.x) > fabsf(n.y)) {
            float inv_len = 1.f / sqrtf(n.x * n.x + n.z * n.z);
            t = mk(n.z * inv_len, 0.f, -n.x * inv_len);
        } else {
            float inv_len = 1.f / sqrtf(n.y * n.y + n.z * n.z);
            t = mk(0.f, n.z * inv_len, -n.y * inv_len);
        }
        s = cross(t, n);
    }
    __device__ __forceinline__ f3 to_local(f3 v) const { return mk(dot(v, s), dot(v, n), dot(v, t)); }
    __device__ __forceinline__ f3 to_world(f3 v) const { return s * v.x + n * v.y + t * v.z; }
};

// ------------------------------------------------------------------ Fresnel
// fresnel(cos, ext, int) of src/base/utils.h:153-177; the reference evaluates
// eta*eta*(1. - c*c) in double.
__device__ __forceinline__ float fresnel_ext_int(float ci, float ext_ior, float int_ior) {
    float etai = ext_ior, etat = int_ior;
    if (ext_ior == int_ior) return 0.f;
    if (ci < 0.f) {
        float tmp = etai; etai = etat; etat = tmp;
        ci = -ci;
    }
    float eta = etai / etat;
    float st2 = (float)((double)(eta * eta) * (1.0 - (double)(ci * ci)));
    if (st2 > 1.f) return 1.f;
    float ct = sqrtf(1.f - st2);
    float rs = (etai * ci - etat * ct) / (etai * ci + etat * ct);
    float rp = (etat * ci - etai * ct) / (etat * ci + etai * ct);
    return (rs * rs + rp * rp) / 2.f;
}

// fresnel_refl_dielectric(eta, cos_i[, cos_t]), src/shading/fresnel.h:75-131
__device__ __forceinline__ float fresnel_refl_ct(float eta, float ci, float ct) {
    if (ci == 0.f && ct == 0.f) return 0.f;
    float fp = eta * ct;
    float rp = (ci - fp) / (ci + fp);
    float fs = eta * ci;
    float rs = (ct - fs) / (ct + fs);
    return 0.5f * (rp * rp + rs * rs);
}
__device__ __forceinline__ float fresnel_refl(float eta, float ci) {
    const float si2 = 1.f - sq(ci);
    const float st2 = si2 * sq(eta);
    const float ct2 = 1.f - st2;
    if (ct2 < 0.f) return 1.f;
    return fresnel_refl_ct(eta, ci, sqrtf(ct2));
}
// fresnel_schlick(eta, cos) (fresnel.h:180-183), double like the reference.
__device__ __forceinline__ float fresnel_schlick_eta(float eta, float c) {
    double r = (1.0 - (double)eta) / (1.0 + (double)eta);
    double F0 = r * r;
    double x = 1.0 - (double)c;
    double x2 = x * x;
    return (float)(F0 + (1.0 - F0) * (x2 * x2 * x));
}
// schlick_weight (fresnel.h:176-178): clamp(1 - cos, 0, 1)^5
__device__ __forceinline__ float schlick_weight(float c) {
    double x = fmin(fmax(1.0 - (double)c, 0.0), 1.0);
    double x2 = x * x;
    return (float)(x2 * x2 * x);
}

// ------------------------------------------------------------------ microfacet
struct Mdf {
    int dist;  // KZ_DIST_GGX / KZ_DIST_BECKMANN
    f3 wi;
    float ax, ay;

    __device__ __forceinline__ float lambda(f3 m) const {
        float c = m.y;
        if (c == 0.f) return 0.f;
        float s = sqrtf(fmaxf(0.f, 1.f - sq(c)));
        if (s == 0.f) return 0.f;
        float alpha;
        if (ax == ay) alpha = ax;
        else alpha = sqrtf(sq((m.x * ax) / s) + sq((m.z * ay) / s));
        float a_rcp = alpha * fabsf(s / c);
        if (dist == KZ_DIST_GGX) return (-1.f + sqrtf(1.f + sq(a_rcp))) * 0.5f;
        float a = 1.f / a_rcp;
        if (a < 1.6f) {
            float a2 = sq(a);
            return (1.f - 1.259f * a + 0.396f * a2) / (3.535f * a + 2.181f * a2);
        }
        return 0.f;
    }
    __device__ __forceinline__ float G(f3 wo) const { return 1.f / (lambda(wi) + lambda(wo) + 1.f); }
    __device__ __forceinline__ float G1(f3 w) const { return 1.f / (lambda(w) + 1.f); }
    __device__ __forceinline__ float D(f3 m) const {
        float c = m.y;
        if (c == 0.f) return dist == KZ_DIST_BECKMANN ? 0.f : sq(ax) * kInvPi;
        float c2 = sq(c);
        float s = sqrtf(fmaxf(0.f, 1.f - c2));
        float c4 = sq(c2);
        float tan2 = (1.f - c2) / c2;
        float A = (ax == ay) ? 1.f / sq(ax) : sq(m.x / (s * ax)) + sq(m.z / (s * ay));
        float x = tan2 * A;
        float Dv;
        if (dist == KZ_DIST_GGX) {
            float tmp = 1 + x;
            Dv = 1.f / (kPi * tmp * tmp);
        } else {
            Dv = kInvPi * expf(-x);
        }
        return Dv / (c4 * ax * ay);
    }
    // visible-normal pdf of m, measure of m (microfacet.h:227-241)
    __device__ __forceinline__ float pdf(f3 m) const {
        float c = wi.y;
        if (c == 0.f) return 0.f;
        return G1(wi) * fabsf(dot(wi, m)) * D(m) / fabsf(c);
    }
};

// Visible-normal sampling. GGX: the exact construction of E. Heitz, "Sampling
// the GGX Distribution of Visible Normals", JCGT 7(4), 2018. Beckmann: stretch,
// sample the standard visible slope by Newton-bisection on its CDF in the erf
// domain (E. Heitz & E. d'Eon, "Importance Sampling Microfacet-Based BSDFs
// using the Distribution of Visible Normals", EGSR 2014), rotate, unstretch.
__device__ __forceinline__ f3 sample_vndf(int dist, f3 wi, float ax, float ay, float u1, float u2) {
    if (dist == KZ_DIST_GGX) {
        f3 V = mk(wi.x, wi.z, wi.y);  // z-up working frame
        f3 Vh = normalize(mk(ax * V.x, ay * V.y, V.z));
        float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
        f3 T1 = lensq > 0.f ? mk(-Vh.y, Vh.x, 0.f) * (1.f / sqrtf(lensq)) : mk(1.f, 0.f, 0.f);
        f3 T2 = cross(Vh, T1);
        float r = sqrtf(u1);
        float phi = 2.f * kPi * u2;
        float sp, cp;
        sincosf(phi, &sp, &cp);
        float t1 = r * cp;
        float t2 = r * sp;
        float s = 0.5f * (1.f + Vh.z);
        t2 = (1.f - s) * sqrtf(1.f - t1 * t1) + s * t2;
        f3 Nh = T1 * t1 + T2 * t2 + Vh * sqrtf(fmaxf(0.f, 1.f - t1 * t1 - t2 * t2));
        f3 Ne = normalize(mk(ax * Nh.x, ay * Nh.y, fmaxf(0.f, Nh.z)));
        return mk(Ne.x, Ne.z, Ne.y);
    }
    f3 ws = normalize(mk(wi.x * ax, wi.y, wi.z * ay));
    float cos_t = ws.y;
    float sin_t = sqrtf(fmaxf(0.f, 1.f - cos_t * cos_t));
    float sx, sy;
    if (cos_t > 0.99999f) {
        double r = sqrt(-log(fmax(1e-12, 1.0 - (double)u1)));
        double p = 2.0 * 3.14159265358979323846 * (double)u2;
        sx = (float)(r * cos(p));
        sy = (float)(r * sin(p));
    } else {
        double tan_t = (double)sin_t / cos_t, cot_t = (double)cos_t / sin_t;
        double c = erf(cot_t);
        double K = tan_t * 0.56418958354775628695;  // 1/sqrt(pi)
        double Z = 1.0 + c + K * exp(-cot_t * cot_t);
        double lo = -1.0, hi = c;
        double uu = fmin(fmax((double)u1, 1e-7), 1.0 - 1e-7);
        double b = -1.0 + uu * (c + 1.0);
        for (int it = 0; it < 40; ++it) {
            if (!(b > lo && b < hi)) b = 0.5 * (lo + hi);
            double ei = erfinv(b);
            double val = (1.0 + b + K * exp(-ei * ei)) / Z - uu;
            if (fabs(val) < 1e-9) break;
            if (val > 0) hi = b; else lo = b;
            b -= val / ((1.0 - ei * tan_t) / Z);
        }
        sx = (float)erfinv(b);
        sy = (float)erfinv(2.0 * fmin(fmax((double)u2, 1e-7), 1.0 - 1e-7) - 1.0);
    }
    float cp = 1.f, sp = 0.f;
    if (sin_t != 0.f) {
        float phi = atan2f(ws.z, ws.x);
        sincosf(phi, &sp, &cp);
    }
    float rx = cp * sx - sp * sy;
    float ry = sp * sx + cp * sy;
    return normalize(mk(-rx * ax, 1.f, -ry * ay));
}

__device__ __forceinline__ f3 reflect_n(f3 wi, f3 n) { return -wi + 2.f * dot(wi, n) * n; }
// refract(wi, n, eta), src/base/utils.h:142-151
__device__ __forceinline__ f3 refract_u(f3 wi, f3 n, float eta) {
    float ci = dot(n, wi);
    if (ci < 0) eta = 1.f / eta;
    float co2 = 1 - (1 - ci * ci) * (eta * eta);
    if (co2 <= 0.f) return mk(0.f, 0.f, 0.f);
    float sign = ci >= 0.f ? 1.f : -1.f;
    return n * (-ci * eta + sign * sqrtf(co2)) + wi * eta;
}

// ------------------------------------------------------------------ lobes
// lobe_eval and lobe_sample stay out of line: one copy of the 21-way lobe
// switch per kernel instead of one per call site (the shading kernels call
// them from three loops). Measured on the terrain frame: shading 42.1 ->
// 40.4 ms, the instruction-cache stalls being the shading kernel's first. A
// translation unit that defines KZ_LOBE_INLINE inlines them instead.
#ifdef KZ_LOBE_INLINE
#define KZ_LOBE_FN __device__ inline
#else
#define KZ_LOBE_FN static __device__ __noinline__
#endif

struct LobeEval {
    f3 f;
    float pdf;
};
struct LobeSample {
    f3 wo;
    f3 weight;
    float pdf;
    bool valid, delta;
};

__device__ __forceinline__ bool lobe_is_delta(uint32_t id) {
    return id == KZ_CLOSURE_KP_MIRROR || id == KZ_CLOSURE_KP_DIELECTRIC || id == KZ_CLOSURE_REFLECTION ||
           id == KZ_CLOSURE_REFRACTION || id == KZ_CLOSURE_TRANSPARENT;
}

// ------------------------------------------------------------------ helpers of the further lobes
__device__ __forceinline__ float pow5(float x) {
    const float x2 = x * x;
    return x2 * x2 * x;
}
// Cosine-weighted direction about +y (Malley's method: a uniform disk
// point lifted onto the hemisphere); pdf y / pi.
__device__ __forceinline__ f3 cosine_hemisphere(float u0, float u1) {
    float r = sqrtf(u0);
    float sp, cp;
    sincosf(2.f * kPi * u1, &sp, &cp);
    float x = r * cp, z = r * sp;
    float y = sqrtf(fmaxf(0.f, 1.f - x * x - z * z));
    return mk(x, y, z);
}
// Orthonormal basis (b1, b2) completing the unit vector n: Duff et al.,
// "Building an Orthonormal Basis, Revisited", JCGT 6(1), 2017.
__device__ __forceinline__ void onb(f3 n, f3& b1, f3& b2) {
    const float sign = n.z >= 0.f ? 1.f : -1.f;
    const float a = -1.f / (sign + n.z);
    const float b = n.x * n.y * a;
    b1 = mk(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    b2 = mk(b, sign + n.y * n.y * a, -n.y);
}
// Beckmann slope pdf D(m) cos(theta_m) (BeckmannPDF, src/shading/microfacet.cpp:10-23)
__device__ __forceinline__ float beckmann_pdf_m(f3 m, float alpha) {
    const float c = m.y;
    if (c <= 0.f) return 0.f;
    const float a2 = alpha * alpha;
    const float s2 = 1.f - c * c;
    const float t = s2 < 0.f ? 0.f : sqrtf(s2) / c;
    return kInvPi * (expf(-(t * t) / a2) / (a2 * (c * c * c)));
}
// Walter et al. 2007 rational fit of the Beckmann Smith G1 (G1,
// src/shading/microfacet.cpp:25-38)
__device__ __forceinline__ float beckmann_g1_walter(f3 m, f3 v, float alpha) {
    if (dot(v, m) / v.y <= 0.f) return 0.f;
    const float s2 = 1.f - v.y * v.y;
    const float t = s2 < 0.f ? 0.f : sqrtf(s2) / v.y;
    const float b = 1.f / (alpha * t);
    if (b >= 1.6f) return 1.f;
    const float b2 = b * b;
    return (3.535f * b + 2.181f * b2) / (1.f + 2.276f * b + 2.577f * b2);
}
// Ward exponent -tan^2(theta_m) (cos^2 phi_m / ax^2 + sin^2 phi_m / ay^2),
// written without dividing by sin(theta_m).
__device__ __forceinline__ float ward_exponent(f3 m, float ax, float ay) {
    return -(sq(m.x / ax) + sq(m.z / ay)) / sq(m.y);
}
// Clearcoat GGX Smith G1 with the fixed alpha 0.25 (Disney 2012)
__device__ __forceinline__ float clearcoat_g1(float c) {
    const float t2 = (1.f - c * c) / (c * c);
    return 2.f / (1.f + sqrtf(1.f + 0.0625f * t2));
}
// GTR1 (Berry) normal distribution, alpha in (0, 1), at the unit half
// vector m; 1 + (a2 - 1) cos^2 is formed as a2 cos^2 + sin^2 so that a small
// alpha near the peak does not cancel.
__device__ __forceinline__ float gtr1_D(float alpha, f3 m) {
    const float a2 = alpha * alpha;
    return (a2 - 1.f) / (kPi * logf(a2) * (a2 * m.y * m.y + (m.x * m.x + m.z * m.z)));
}

__device__ __forceinline__ Mdf lobe_mdf(const kz_lobe& l, f3 wi, float& eta) {
    Mdf m;
    m.wi = wi;
    if (l.closure_id == KZ_CLOSURE_KP_GLOSS || l.closure_id == KZ_CLOSURE_KP_GLASS) {
        m.dist = (int)l.params[0];
        m.ax = l.params[7];
        m.ay = l.params[8];
        eta = l.params[9];
    } else if (l.closure_id == KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL) {
        m.dist = KZ_DIST_GGX;
        m.ax = l.params[6];
        m.ay = l.params[7];
        eta = l.params[8];
    } else {
        m.dist = KZ_DIST_GGX;
        m.ax = l.params[3];
        m.ay = l.params[4];
        eta = 1.f;
    }
    return m;
}

// Value and pdf of one lobe exactly as the reference eval functions return
// them; a configuration the reference rejects gives (0, 0). kRefNorm selects
// the reference's own normalisation of half vectors (a double-precision
// reciprocal length), used by the reference-convention batch kernel; the
// shading kernels use the float form.
template <bool kRefNorm = false>
__device__ inline LobeEval lobe_eval_reference(const kz_lobe& l, f3 wi, f3 wo) {
    LobeEval r{mk(0.f, 0.f, 0.f), 0.f};
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE: {
        f3 n = mk(l.params[0], l.params[1], l.params[2]);
        float p = fmaxf(dot(wo, n), 0.f) * kInvPi;
        r.f = mk(p, p, p);
        r.pdf = p;
        return r;
    }
    case KZ_CLOSURE_KP_GLOSS: {
        float eta;
        Mdf mdf = lobe_mdf(l, wi, eta);
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return r;
        f3 m = nrm<kRefNorm>(wi + wo);
        if (dot(wo, m) == 0.f) return r;
        float D = mdf.D(m), G = mdf.G(wo);
        float cmi = dot(m, wi);
        float F = fresnel_refl(eta, mdf.dist == KZ_DIST_BECKMANN ? cmi : fabsf(cmi));
        float v = D * G * F / (4.f * ci * co);
        r.f = mk(v, v, v);
        r.pdf = mdf.pdf(m);
        return r;
    }
    case KZ_CLOSURE_KP_GLASS: {
        float eta;
        Mdf mdf = lobe_mdf(l, wi, eta);
        float ci = wi.y, co = wo.y;
        if (eta == 1.f) return r;
        if (ci < 0) eta = 1.f / eta;
        if (ci * co >= 0.f) {
            f3 m = nrm<kRefNorm>(wi + wo);
            float cmi = dot(wi, m);
            float F = fresnel_refl(eta, cmi);
            r.pdf = cmi == 0.f ? 0.f : (1.f / (4.f * fabsf(cmi))) * mdf.pdf(m);
            float denom = fabsf(4.f * wi.y * wo.y);
            float v = denom == 0.f ? 0.f : F * mdf.D(m) * mdf.G(wo) / denom;
            r.f = mk(v, v, v);
        } else {
            f3 m = nrm<kRefNorm>(wi + eta * wo);
            if (m.y < 0.f) m = -m;
            float cmi = dot(wi, m);
            float F = fresnel_refl(eta, cmi);
            float cmo = dot(m, wo);
            float dn = cmi + eta * cmo;
            r.pdf = fabsf(dn) < 1.0e-6f ? 0.f : fabsf(cmo) * sq(eta / dn) * mdf.pdf(m);
            float v = 0.f;
            if (wi.y != 0.f && wo.y != 0.f) {
                float c = fabsf((cmi * cmo) / (wi.y * wo.y));
                float d2 = sq(dn);  // the reference squares twice (bsdfs.h:578-591)
                if (!(fabsf(d2) < 1.0e-6f)) v = c * mdf.D(m) * mdf.G(wo) * (1.f - F) * sq(eta) / sq(d2);
            }
            r.f = mk(v, v, v);
        }
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL: {
        float eta;
        Mdf mdf = lobe_mdf(l, wi, eta);
        float co = wo.y, ci = wi.y;
        if (ci * co < 0.f) return r;
        f3 wh = nrm<kRefNorm>(wi + wo);
        float com = dot(wo, wh);
        if (com == 0.f) return r;
        float D = fminf(4.f, mdf.D(wh));
        float G = mdf.G(wo);
        float s = fresnel_schlick_eta(eta, com);
        float k = D * G / (4.f * ci * co);
        r.f = mk(fminf(1.f, k * (l.params[0] + (1.f - l.params[0]) * s)),
                 fminf(1.f, k * (l.params[1] + (1.f - l.params[1]) * s)),
                 fminf(1.f, k * (l.params[2] + (1.f - l.params[2]) * s)));
        r.pdf = fmaxf(0.f, mdf.pdf(wh));
        return r;
    }
    case KZ_CLOSURE_CONDUCTOR_GGX: {
        float eta;
        Mdf mdf = lobe_mdf(l, wi, eta);
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return r;
        f3 m = nrm<kRefNorm>(wi + wo);
        float com = dot(wo, m);
        if (com <= 0.f) return r;
        float w = schlick_weight(com);
        float k = mdf.D(m) * mdf.G(wo) / (4.f * ci * co);
        r.f = mk(k * (l.params[0] + (1.f - l.params[0]) * w), k * (l.params[1] + (1.f - l.params[1]) * w),
                 k * (l.params[2] + (1.f - l.params[2]) * w));
        r.pdf = mdf.pdf(m);
        return r;
    }
    case KZ_CLOSURE_PHONG: {  // Phong::eval, bsdfs.cpp:43-59 (returns the sample weight)
        const f3 N = mk(l.params[0], l.params[1], l.params[2]);
        const float e = l.params[3];
        const float cni = wo.y, cno = dot(N, wi);
        if (cni > 0.f && cno > 0.f) {
            const f3 R = (2.f * cno) * N - wi;
            const float cri = dot(R, wo);
            if (cri > 0.f) {
                r.pdf = (e + 1.f) * (0.5f * kInvPi) * powf(cri, e);
                const float v = cni * (e + 2.f) / (e + 1.f);
                r.f = mk(v, v, v);
            }
        }
        return r;
    }
    case KZ_CLOSURE_WARD: {  // Ward::eval, bsdfs.cpp:92-112
        const float ax = l.params[6], ay = l.params[7];
        const float ci = wi.y, co = wo.y;
        if (ci <= 0.f || co <= 0.f) return r;
        const f3 m = nrm<kRefNorm>(wi + wo);
        const float sv = sqrtf(fmaxf(0.f, 1.f - ci * ci));
        // stretched_roughness (microfacet.h:60-73) takes sin(theta) of wi here
        const float A = ax == ay ? 1.f / sq(ax) : sq(m.x / (sv * ax)) + sq(m.z / (sv * ay));
        const float t2 = fmaxf(0.f, 1.f - m.y * m.y) / (m.y * m.y);
        const float tmp = expf(-t2 * A) / (4.f * kPi * ax * ay);
        r.pdf = fmaxf(tmp / (dot(m, wi) * (m.y * m.y * m.y)), 0.f);
        const float v = tmp / sqrtf(ci * co);
        r.f = mk(v, v, v);
        return r;
    }
    case KZ_CLOSURE_TRANSPARENT:  // Transparent::eval, bsdfs.cpp:205-209
        r.f = mk(1.f, 1.f, 1.f);
        r.pdf = 1.f;
        return r;
    case KZ_CLOSURE_TRANSLUCENT: {  // Translucent::eval, bsdfs.cpp:219-223
        r.pdf = fmaxf(wo.y, 0.f) * kInvPi;
        r.f = mk(kInvPi, kInvPi, kInvPi);
        return r;
    }
    case KZ_CLOSURE_KP_MICROFACET: {  // KpMicrofacet::eval, bsdfs.cpp:300-319
        const float alpha = l.params[0], kd = l.params[3];
        const float ci = wi.y, co = wo.y;
        if (ci <= 0.f || co <= 0.f) return r;
        const f3 wh = nrm<kRefNorm>(wi + wo);
        const float D = beckmann_pdf_m(wh, alpha);
        const float F = fresnel_ext_int(dot(wh, wi), l.params[2], l.params[1]);
        const float G = beckmann_g1_walter(wh, wi, alpha) * beckmann_g1_walter(wh, wo, alpha);
        const float ks = 1.f - kd;
        const float Jh = 1.f / (4.f * dot(wh, wo));
        r.pdf = ks * D * Jh + kd * co * kInvPi;
        const float v = kInvPi + ks * D * F * G / (4.f * ci * co * wh.y);
        r.f = mk(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE: {  // bsdfs.cpp:563-576: only the view factor survives
        const float ci = wi.y, co = wo.y;
        if (co <= 0.f || ci <= 0.f) return r;
        r.pdf = co * kInvPi;
        const float v = kInvPi * (1.f - 0.5f * pow5(1.f - ci));
        r.f = mk(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_RETRO: {  // bsdfs.cpp:586-605
        const float ci = wi.y, co = wo.y;
        if (co <= 0.f || ci <= 0.f) return r;
        r.pdf = co * kInvPi;
        const float FL = pow5(1.f - co), FV = pow5(1.f - ci);
        const f3 wh = nrm<kRefNorm>(wi + wo);
        const float RR = 2.f * l.params[3] * sq(dot(wo, wh));
        const float v = kInvPi * RR * (FL + FV + FL * FV * (RR - 1.f));
        r.f = mk(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_FAKESS: {  // bsdfs.cpp:614-640 (no hemisphere test)
        const f3 wh = nrm<kRefNorm>(wi + wo);
        const float fss90 = sq(dot(wh, wo)) * l.params[0];
        const float aci = fabsf(wi.y), aco = fabsf(wo.y);
        const float fi = pow5(1.f - aci), fo = pow5(1.f - aco);
        const float fss = (1.f + fi * (fss90 - 1.f)) * (1.f + fo * (fss90 - 1.f));
        const float ss = 1.25f * (fss * (1.f / (aci + aco) - 0.5f) + 0.5f);
        r.pdf = fmaxf(wo.y, 0.f) * kInvPi;
        const float v = ss * kInvPi;
        r.f = mk(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_SHEEN: {  // bsdfs.cpp:649-666
        const float ci = wi.y, co = wo.y;
        if (co <= 0.f || ci <= 0.f) return r;
        r.pdf = co * kInvPi;
        const f3 wh = nrm<kRefNorm>(wi + wo);
        const float cv = dot(wh, wo);
        const float v = cv < 1e-6f ? l.params[3] : l.params[3] * pow5(1.f - cv);
        r.f = mk(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT: {  // bsdfs.cpp:736-780: D takes cos, G1 takes tan
        const float ci = wi.y, co = wo.y;
        if (ci <= 0.f || co <= 0.f) return r;
        const f3 wh = nrm<kRefNorm>(wi + wo);
        const float ch = wh.y;
        const float a2 = sq(l.params[3]);
        const float D = (a2 - 1.f) / (kPi * logf(a2) * (1.f + (a2 - 1.f) * ch));
        const float ti = sqrtf(fmaxf(0.f, 1.f - ci * ci)) / ci, to = sqrtf(fmaxf(0.f, 1.f - co * co)) / co;
        const float G = (2.f / (1.f + sqrtf(1.f + 0.0625f * ti))) * (2.f / (1.f + sqrtf(1.f + 0.0625f * to)));
        const float F = 0.04f + 0.96f * pow5(1.f - ci);
        r.pdf = fmaxf(0.f, D * ch / (4.f * dot(wo, wh)));
        const float v = fminf(fmaxf(D * G * F * 0.25f, 0.f), 0.25f);
        r.f = mk(v, v, v);
        return r;
    }
    default:  // KpMirror, KpDielectric, Reflection, Refraction (delta: eval 0, pdf 0) and Le-only ids
        return r;
    }
}

// f*|cos(wo)| and the solid-angle pdf of wo under the lobe's own sampler.
KZ_LOBE_FN LobeEval lobe_eval(const kz_lobe& l, f3 wi, f3 wo) {
    LobeEval z{mk(0.f, 0.f, 0.f), 0.f};
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE:
        return lobe_eval_reference(l, wi, wo);
    case KZ_CLOSURE_KP_GLOSS:
    case KZ_CLOSURE_CONDUCTOR_GGX:
    case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL: {
        LobeEval r = lobe_eval_reference(l, wi, wo);
        if (r.pdf == 0.f || wi.y <= 0.f || wo.y <= 0.f) return z;
        f3 m = normalize(wi + wo);
        float wom = fabsf(dot(wo, m));
        if (wom == 0.f) return z;
        r.pdf = r.pdf / (4.f * wom);
        r.f = r.f * fabsf(wo.y);
        return r;
    }
    case KZ_CLOSURE_KP_GLASS: {
        LobeEval r = lobe_eval_reference(l, wi, wo);
        float eta = l.params[9];
        if (eta == 1.f) return z;
        if (wi.y < 0) eta = 1.f / eta;
        f3 m;
        bool refl = wi.y * wo.y >= 0.f;
        if (refl) {
            m = normalize(wi + wo);
        } else {
            m = normalize(wi + eta * wo);
            if (m.y < 0.f) m = -m;
        }
        float F = fresnel_refl(eta, fminf(fmaxf(dot(m, wi), -1.f), 1.f));
        r.pdf *= refl ? F : (1.f - F);
        r.f = r.f * fabsf(wo.y);
        return r;
    }
    case KZ_CLOSURE_PHONG: {  // modified Phong, f = (e+2)/(2 pi) cos_r^e, sampled about R
        const f3 N = mk(l.params[0], l.params[1], l.params[2]);
        const float e = l.params[3];
        const float cno = dot(N, wi), cni = dot(N, wo);
        if (cno <= 0.f || cni <= 0.f) return z;
        const float cri = dot((2.f * cno) * N - wi, wo);
        if (cri <= 0.f) return z;
        const float lobe = powf(cri, e) * (0.5f * kInvPi);
        const float v = (e + 2.f) * lobe * cni;
        return LobeEval{mk(v, v, v), (e + 1.f) * lobe};
    }
    case KZ_CLOSURE_WARD: {  // Walter, "Notes on the Ward BRDF" (2005), eqs. 3 and 9
        const float ax = l.params[6], ay = l.params[7];
        const float ci = wi.y, co = wo.y;
        if (ci <= 0.f || co <= 0.f) return z;
        const f3 m = normalize(wi + wo);
        const float k = expf(ward_exponent(m, ax, ay)) / (4.f * kPi * ax * ay);
        const float v = k * co / sqrtf(ci * co);
        return LobeEval{mk(v, v, v), k / (dot(m, wi) * (m.y * m.y * m.y))};
    }
    case KZ_CLOSURE_TRANSLUCENT: {  // Lambertian transmission: wo on the far side of wi
        if (wi.y * wo.y >= 0.f) return z;
        const float v = fabsf(wo.y) * kInvPi;
        return LobeEval{mk(v, v, v), v};
    }
    case KZ_CLOSURE_KP_MICROFACET: {  // Cook-Torrance (Beckmann) + kd/pi, sampled by ks : kd
        const float alpha = l.params[0], kd = l.params[3];
        const float ci = wi.y, co = wo.y;
        if (ci <= 0.f || co <= 0.f) return z;
        const f3 wh = normalize(wi + wo);
        const float D = beckmann_pdf_m(wh, alpha);
        const float F = fresnel_ext_int(dot(wh, wi), l.params[2], l.params[1]);
        const float G = beckmann_g1_walter(wh, wi, alpha) * beckmann_g1_walter(wh, wo, alpha);
        const float ks = 1.f - kd;
        const float v = (kd * kInvPi + ks * D * F * G / (4.f * ci * co * wh.y)) * co;
        return LobeEval{mk(v, v, v), ks * D / (4.f * dot(wh, wo)) + kd * co * kInvPi};
    }
    case KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE: {  // Burley 2015: (1 - F_L / 2)(1 - F_V / 2) / pi
        const float ci = wi.y, co = wo.y;
        if (co <= 0.f || ci <= 0.f) return z;
        const float v = kInvPi * (1.f - 0.5f * pow5(1.f - co)) * (1.f - 0.5f * pow5(1.f - ci)) * co;
        return LobeEval{mk(v, v, v), co * kInvPi};
    }
    case KZ_CLOSURE_KP_PRINCIPLE_RETRO:
    case KZ_CLOSURE_KP_PRINCIPLE_SHEEN: {  // reference f times cos, cosine-sampled
        if (wi.y <= 0.f || wo.y <= 0.f) return z;
        LobeEval r = lobe_eval_reference(l, wi, wo);
        r.f = r.f * wo.y;
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_FAKESS: {  // reflection only
        if (wi.y <= 0.f || wo.y <= 0.f) return z;
        LobeEval r = lobe_eval_reference(l, wi, wo);
        r.f = r.f * wo.y;
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT: {  // Disney 2012 clearcoat: GTR1, Smith G (alpha 0.25), F0 0.04
        const float ci = wi.y, co = wo.y;
        if (ci <= 0.f || co <= 0.f) return z;
        const f3 wh = normalize(wi + wo);
        const float cd = dot(wo, wh);
        if (cd <= 0.f) return z;
        const float D = gtr1_D(l.params[3], wh);
        const float F = 0.04f + 0.96f * pow5(1.f - cd);
        const float v = 0.25f * D * F * clearcoat_g1(ci) * clearcoat_g1(co) / (4.f * ci);
        return LobeEval{mk(v, v, v), D * wh.y / (4.f * cd)};
    }
    default:  // delta lobes and Le-only ids
        return z;
    }
}

KZ_LOBE_FN LobeSample lobe_sample(const kz_lobe& l, f3 wi, float u0, float u1, float u2) {
    LobeSample s{mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f), 0.f, false, false};
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE:
    case KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE:
    case KZ_CLOSURE_KP_PRINCIPLE_RETRO:
    case KZ_CLOSURE_KP_PRINCIPLE_FAKESS:
    case KZ_CLOSURE_KP_PRINCIPLE_SHEEN:
    case KZ_CLOSURE_TRANSLUCENT: {
        s.wo = cosine_hemisphere(u0, u1);
        if (l.closure_id == KZ_CLOSURE_TRANSLUCENT) {
            if (wi.y == 0.f) return s;
            if (wi.y > 0.f) s.wo.y = -s.wo.y;
        }
        LobeEval e = lobe_eval(l, wi, s.wo);
        if (e.pdf <= 0.f) return s;
        s.pdf = e.pdf;
        s.weight = e.f * (1.f / e.pdf);
        s.valid = true;
        return s;
    }
    case KZ_CLOSURE_KP_MIRROR:
        s.wo = reflect_n(wi, mk(0.f, 1.f, 0.f));
        s.weight = mk(1.f, 1.f, 1.f);
        s.valid = s.delta = true;
        return s;
    case KZ_CLOSURE_KP_DIELECTRIC: {
        float ior_in = l.params[0], ior_ex = l.params[1];
        f3 n = mk(0.f, 1.f, 0.f);
        float ci = dot(wi, n);
        float F = fresnel_ext_int(ci, ior_ex, ior_in);
        if (u0 < F) {
            s.wo = reflect_n(wi, n);
        } else {
            float fac = ior_in / ior_ex;
            if (ci < 0.f) {
                fac = ior_ex / ior_in;
                n = -n;
            }
            s.wo = refract_u(-wi, n, fac);
            if (is_zero(s.wo)) return s;
        }
        s.weight = mk(1.f, 1.f, 1.f);
        s.valid = s.delta = true;
        return s;
    }
    case KZ_CLOSURE_REFLECTION:  // Reflection::sample, bsdfs.cpp:150-167 (no Fresnel factor)
        if (wi.y <= 0.f) return s;
        s.wo = reflect_n(wi, mk(0.f, 1.f, 0.f));
        s.weight = mk(1.f, 1.f, 1.f);
        s.valid = s.delta = true;
        return s;
    case KZ_CLOSURE_REFRACTION: {  // Snell transmission through the surface, eta = inside / outside
        f3 n = mk(0.f, 1.f, 0.f);
        float fac = l.params[3];
        if (wi.y < 0.f) {
            fac = 1.f / fac;
            n = -n;
        }
        s.wo = refract_u(-wi, n, fac);
        if (is_zero(s.wo)) return s;
        s.weight = mk(1.f, 1.f, 1.f);
        s.valid = s.delta = true;
        return s;
    }
    case KZ_CLOSURE_TRANSPARENT:  // Transparent::sample, bsdfs.cpp:211-217: straight through
        s.wo = -wi;
        s.weight = mk(1.f, 1.f, 1.f);
        s.valid = s.delta = true;
        return s;
    case KZ_CLOSURE_PHONG:
    case KZ_CLOSURE_WARD:
    case KZ_CLOSURE_KP_MICROFACET:
    case KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT: {
        if (wi.y <= 0.f) return s;
        if (l.closure_id == KZ_CLOSURE_PHONG) {
            // cos^e lobe about the mirror direction R
            const f3 N = mk(l.params[0], l.params[1], l.params[2]);
            const float cno = dot(N, wi);
            if (cno <= 0.f) return s;
            const f3 R = (2.f * cno) * N - wi;
            f3 b1, b2;
            onb(R, b1, b2);
            const float ct = powf(u1, 1.f / (l.params[3] + 1.f));
            const float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
            float sp, cp;
            sincosf(2.f * kPi * u0, &sp, &cp);
            s.wo = b1 * (st * cp) + b2 * (st * sp) + R * ct;
        } else {
            f3 m;
            if (l.closure_id == KZ_CLOSURE_WARD) {
                // Walter's notes eqs. 6-7: phi from the stretched angle, quadrant kept
                const float ax = l.params[6], ay = l.params[7];
                float sp, cp;
                sincosf(2.f * kPi * u0, &sp, &cp);
                const float px = ax * cp, pz = ay * sp;
                const float inv = 1.f / sqrtf(px * px + pz * pz);
                const float cphi = px * inv, sphi = pz * inv;
                const float A = sq(cphi / ax) + sq(sphi / ay);
                const float t = sqrtf(-logf(1.f - u1) / A);
                const float ct = 1.f / sqrtf(1.f + t * t);
                m = mk(t * ct * cphi, ct, t * ct * sphi);
            } else if (l.closure_id == KZ_CLOSURE_KP_MICROFACET) {
                if (u2 >= 1.f - l.params[3]) {  // diffuse part, probability kd
                    s.wo = cosine_hemisphere(u0, u1);
                    m = mk(0.f, 0.f, 0.f);
                } else {  // Beckmann normal, BeckmannMDF (microfacet.cpp:3-8)
                    const float t = sqrtf(-sq(l.params[0]) * logf(1.f - u1));
                    const float ct = 1.f / sqrtf(1.f + t * t);
                    float sp, cp;
                    sincosf(2.f * kPi * u0, &sp, &cp);
                    m = mk(t * ct * cp, ct, t * ct * sp);
                }
            } else {  // GTR1 half vector, Burley 2012 appendix B
                const float a2 = sq(l.params[3]);
                const float ct = sqrtf(fmaxf(0.f, (1.f - powf(a2, 1.f - u1)) / (1.f - a2)));
                const float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
                float sp, cp;
                sincosf(2.f * kPi * u0, &sp, &cp);
                m = mk(st * cp, ct, st * sp);
            }
            if (!is_zero(m)) s.wo = reflect_n(wi, m);
        }
        if (s.wo.y <= 0.f) return s;
        LobeEval e = lobe_eval(l, wi, s.wo);
        if (e.pdf <= 0.f) return s;
        s.pdf = e.pdf;
        s.weight = e.f * (1.f / e.pdf);
        s.valid = true;
        return s;
    }
    case KZ_CLOSURE_KP_GLOSS:
    case KZ_CLOSURE_CONDUCTOR_GGX:
    case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL: {
        if (wi.y <= 0.f) return s;
        float eta;
        Mdf mdf = lobe_mdf(l, wi, eta);
        f3 m = sample_vndf(mdf.dist, wi, mdf.ax, mdf.ay, u0, u1);
        s.wo = reflect_n(wi, m);
        if (s.wo.y <= 0.f) return s;
        LobeEval e = lobe_eval(l, wi, s.wo);
        if (e.pdf <= 0.f) return s;
        s.pdf = e.pdf;
        s.weight = e.f * (1.f / e.pdf);
        s.valid = true;
        return s;
    }
    case KZ_CLOSURE_KP_GLASS: {
        float eta;
        Mdf mdf = lobe_mdf(l, wi, eta);
        if (eta == 1.f) return s;
        if (wi.y < 0.f) eta = 1.f / eta;
        f3 wis = wi.y < 0.f ? -wi : wi;
        f3 m = sample_vndf(mdf.dist, wis, mdf.ax, mdf.ay, u0, u1);
        float cmi = fminf(fmaxf(dot(m, wi), -1.f), 1.f);
        float F = fresnel_refl(eta, cmi);
        if (u2 < F) {
            s.wo = reflect_n(wi, m);
            if (wi.y * s.wo.y <= 0.f) return s;
        } else {
            s.wo = refract_u(wi, m, eta);
            if (is_zero(s.wo) || wi.y * s.wo.y > 0.f) return s;
            s.wo = normalize(s.wo);
        }
        LobeEval e = lobe_eval(l, wi, s.wo);
        if (e.pdf <= 0.f) return s;
        s.pdf = e.pdf;
        s.weight = e.f * (1.f / e.pdf);
        s.valid = true;
        return s;
    }
    default:
        return s;
    }
}

__device__ __forceinline__ float power_heuristic(float f, float g) { return (f * f) / (f * f + g * g); }

}  // namespace kz
