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
    return id == KZ_CLOSURE_KP_MIRROR || id == KZ_CLOSURE_KP_DIELECTRIC;
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
// them; a configuration the reference rejects gives (0, 0).
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
        f3 m = normalize(wi + wo);
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
            f3 m = normalize(wi + wo);
            float cmi = dot(wi, m);
            float F = fresnel_refl(eta, cmi);
            r.pdf = cmi == 0.f ? 0.f : (1.f / (4.f * fabsf(cmi))) * mdf.pdf(m);
            float denom = fabsf(4.f * wi.y * wo.y);
            float v = denom == 0.f ? 0.f : F * mdf.D(m) * mdf.G(wo) / denom;
            r.f = mk(v, v, v);
        } else {
            f3 m = normalize(wi + eta * wo);
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
        f3 wh = normalize(wi + wo);
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
        f3 m = normalize(wi + wo);
        float com = dot(wo, m);
        if (com <= 0.f) return r;
        float w = schlick_weight(com);
        float k = mdf.D(m) * mdf.G(wo) / (4.f * ci * co);
        r.f = mk(k * (l.params[0] + (1.f - l.params[0]) * w), k * (l.params[1] + (1.f - l.params[1]) * w),
                 k * (l.params[2] + (1.f - l.params[2]) * w));
        r.pdf = mdf.pdf(m);
        return r;
    }
    default:  // KpMirror, KpDielectric (delta: eval 0, pdf 0) and Le-only ids
        return r;
    }
}

// f*|cos(wo)| and the solid-angle pdf of wo under the lobe's own sampler.
__device__ inline LobeEval lobe_eval(const kz_lobe& l, f3 wi, f3 wo) {
    LobeEval r = lobe_eval_reference(l, wi, wo);
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE:
        return r;
    case KZ_CLOSURE_KP_GLOSS:
    case KZ_CLOSURE_CONDUCTOR_GGX:
    case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL: {
        LobeEval z{mk(0.f, 0.f, 0.f), 0.f};
        if (r.pdf == 0.f || wi.y <= 0.f || wo.y <= 0.f) return z;
        f3 m = normalize(wi + wo);
        float wom = fabsf(dot(wo, m));
        if (wom == 0.f) return z;
        r.pdf = r.pdf / (4.f * wom);
        r.f = r.f * fabsf(wo.y);
        return r;
    }
    case KZ_CLOSURE_KP_GLASS: {
        float eta = l.params[9];
        if (eta == 1.f) return LobeEval{mk(0.f, 0.f, 0.f), 0.f};
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
    default:
        return LobeEval{mk(0.f, 0.f, 0.f), 0.f};
    }
}

__device__ inline LobeSample lobe_sample(const kz_lobe& l, f3 wi, float u0, float u1, float u2) {
    LobeSample s{mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f), 0.f, false, false};
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE: {
        float r = sqrtf(u0);
        float sp, cp;
        sincosf(2.f * kPi * u1, &sp, &cp);
        float x = r * cp, z = r * sp;
        float y = sqrtf(fmaxf(0.f, 1.f - x * x - z * z));
        s.wo = mk(x, y, z);
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
