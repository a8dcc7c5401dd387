// Golden-vector harness over kazen_proto's own header-only closure math.
//
// TEST INFRASTRUCTURE: compiled by oracle/ref_build.py from the reference's
// headers where they lie (src/shading/microfacet.h, src/shading/fresnel.h,
// src/base/utils.h, src/core/sampling.h, src/base/vec.h) plus the stand-ins
// in oracle/ref_shim for their third-party includes; its output becomes the
// fixture tests/golden/reference_closure_vectors.npz. Nothing here is part of
// the product.
//
// Every emitted value is computed by the reference's own functions:
// MicrofacetInterface<GGXDist | BeckmannDist>::D / lambda / G1 / G / pdf
// (microfacet.h:95-291), fresnel_dielectric / fresnel_refl_dielectric /
// fresnel_trans_dielectric / fresnel_schlick / schlick_weight (fresnel.h:12-187),
// fresnel / refract / Frame (utils.h:133-210), to_uniform_disk /
// to_cosine_hemisphere / sample_hemisphere / power_heuristic (sampling.h:25-108).
// Three closure evals are composed from those functions in the order of the
// reference's closure code: KpGloss::eval (bsdfs.cpp:359-392),
// KpPrincipleSpecularReflection::eval (bsdfs.cpp:688-717) and Diffuse::eval
// (bsdfs.cpp:27-33), which cannot be compiled as they stand (they read OSL's
// shading context).
//
// Output: text, one table per "# name ncols" header line, then one row of
// space-separated %.9g values per case.
#include <cmath>
#include <cstdint>
#include <cstdio>

// OIIO::fast_exp is reached only by BeckmannDist::sample_slope
// (microfacet.h:169), which no emitted value calls; the exact exp stands in.
namespace OIIO {
inline float fast_exp(float x) { return std::exp(x); }
}  // namespace OIIO

#include "core/sampling.h"
#include "shading/fresnel.h"
#include "shading/microfacet.h"

namespace {

// splitmix64: the harness's own input generator
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }
    float range(float a, float b) { return a + (b - a) * uniform(); }
};

Vec3f unit(Rng& r) {
    for (;;) {
        float x = r.range(-1.f, 1.f), y = r.range(-1.f, 1.f), z = r.range(-1.f, 1.f);
        float l2 = x * x + y * y + z * z;
        if (l2 > 1e-4f && l2 <= 1.f) {
            float il = 1.f / std::sqrt(l2);
            return Vec3f(x * il, y * il, z * il);
        }
    }
}

// an upper-hemisphere direction; one in ten grazing (cos theta < 1e-3)
Vec3f upper(Rng& r, int k) {
    Vec3f v = unit(r);
    if (v[1] < 0.f) v[1] = -v[1];
    if (k % 10 == 3) {
        v[1] = r.range(1e-5f, 1e-3f);
        float s = std::sqrt(std::max(0.f, 1.f - v[1] * v[1])) / std::sqrt(v[0] * v[0] + v[2] * v[2]);
        v[0] *= s;
        v[2] *= s;
    }
    return v;
}

void row(std::initializer_list<float> vals) {
    bool first = true;
    for (float v : vals) {
        std::printf(first ? "%.9g" : " %.9g", (double)v);
        first = false;
    }
    std::printf("\n");
}

template <typename MDF>
void mdf_table(const char* name, Rng& r, int n) {
    // wi wo m ax ay -> D(m) lambda(wi) lambda(wo) G1(wi) G1(wo) G(wo) pdf(m)
    std::printf("# %s 18\n", name);
    for (int k = 0; k < n; ++k) {
        Vec3f wi = upper(r, k), wo = (k % 4 == 1) ? unit(r) : upper(r, k + 1);
        float ax = r.range(0.02f, 1.f), ay = (k % 2) ? r.range(0.02f, 1.f) : ax;
        Vec3f m = (k % 5 == 4) ? upper(r, k + 2) : base::normalize(wi + wo);
        MicrofacetInterface<MDF> mdf(wi, ax, ay);
        row({wi[0], wi[1], wi[2], wo[0], wo[1], wo[2], m[0], m[1], m[2], ax, ay, mdf.D(m), mdf.lambda(wi),
             mdf.lambda(wo), mdf.G1(wi), mdf.G1(wo), mdf.G(wo), mdf.pdf(m)});
    }
}

// KpGloss::eval (bsdfs.cpp:359-392) on the reference's functions; dist 0 = GGX, 1 = Beckmann
void kpgloss_table(Rng& r, int n) {
    // dist wi wo ax ay eta -> f pdf
    std::printf("# kpgloss 12\n");
    for (int k = 0; k < n; ++k) {
        int dist = k & 1;
        Vec3f wi = upper(r, k), wo = (k % 7 == 2) ? unit(r) : upper(r, k + 1);
        float ax = r.range(0.02f, 1.f), ay = (k % 3) ? r.range(0.02f, 1.f) : ax, eta = r.range(0.3f, 2.5f);
        float f = 0.f, pdf = 0.f;
        float ci = cos_theta(wi), co = cos_theta(wo);
        if (ci > 0 && co > 0) {
            const Vec3f m = base::normalize(wi + wo);
            if (base::dot(wo, m) != 0.f) {
                float D, G, F;
                if (dist == 1) {
                    auto mdf = MicrofacetInterface<BeckmannDist>(wi, ax, ay);
                    D = mdf.D(m);
                    G = mdf.G(wo);
                    F = fresnel_refl_dielectric(eta, base::dot(m, wi));
                    pdf = mdf.pdf(m);
                } else {
                    auto mdf = MicrofacetInterface<GGXDist>(wi, ax, ay);
                    D = mdf.D(m);
                    G = mdf.G(wo);
                    F = fresnel_refl_dielectric(eta, std::abs(base::dot(m, wi)));
                    pdf = mdf.pdf(m);
                }
                f = D * G * F / (4.f * ci * co);
            }
        }
        row({(float)dist, wi[0], wi[1], wi[2], wo[0], wo[1], wo[2], ax, ay, eta, f, pdf});
    }
}

// KpPrincipleSpecularReflection::eval (bsdfs.cpp:688-717), N = +y
void principle_specular_table(Rng& r, int n) {
    // wi wo ax ay eta F0rgb -> f rgb, pdf
    std::printf("# principle_specular 16\n");
    const Vec3f nrm(0.f, 1.f, 0.f);
    for (int k = 0; k < n; ++k) {
        Vec3f wi = upper(r, k), wo = (k % 7 == 2) ? unit(r) : upper(r, k + 1);
        float ax = r.range(0.02f, 1.f), ay = (k % 3) ? r.range(0.02f, 1.f) : ax, eta = r.range(1.05f, 2.5f);
        Vec3f F0(r.uniform(), r.uniform(), r.uniform());
        RGBSpectrum f(0.f);
        float pdf = 0.f;
        float co = base::dot(nrm, wo), ci = base::dot(nrm, wi);
        if (!(ci * co < 0.)) {
            const Vec3f wh = base::normalize(wi + wo);
            float cos_om = base::dot(wo, wh);
            if (cos_om != 0.f) {
                auto mdf = MicrofacetInterface<GGXDist>(wi, ax, ay);
                auto D = std::min(4.f, mdf.D(wh));
                auto G = mdf.G(wo);
                auto F = base::lerp(F0, RGBSpectrum{1}, RGBSpectrum(fresnel_schlick(eta, cos_om)));
                pdf = std::max(0.f, mdf.pdf(wh));
                f = base::vec_min(RGBSpectrum{1.f}, D * G * F / (4.f * ci * co));
            }
        }
        row({wi[0], wi[1], wi[2], wo[0], wo[1], wo[2], ax, ay, eta, F0[0], F0[1], F0[2], f[0], f[1], f[2], pdf});
    }
}

// Diffuse::eval (bsdfs.cpp:27-33), N = +y: value = pdf = max(wo . N, 0) / pi
void diffuse_table(Rng& r, int n) {
    std::printf("# diffuse 4\n");
    const Vec3f nrm(0.f, 1.f, 0.f);
    for (int k = 0; k < n; ++k) {
        Vec3f wo = unit(r);
        float pdf = std::max(base::dot(wo, nrm), 0.f) * constants::one_div_pi<float>();
        row({wo[0], wo[1], wo[2], pdf});
    }
}

void fresnel_table(Rng& r, int n) {
    // cos eta ext int -> fresnel_dielectric(cos, eta) fresnel_refl_dielectric(eta, |cos|)
    //   fresnel_trans_dielectric(eta, |cos|) fresnel(cos, ext, int) fresnel_schlick(eta, |cos|) schlick_weight(|cos|)
    std::printf("# fresnel 10\n");
    for (int k = 0; k < n; ++k) {
        float c = r.range(-1.f, 1.f);
        if (k % 11 == 5) c = r.range(-1e-3f, 1e-3f);
        float eta = r.range(0.3f, 2.5f), ext = r.range(1.f, 1.1f), in = r.range(1.1f, 2.f);
        float ac = std::fabs(c);
        row({c, eta, ext, in, fresnel_dielectric(c, eta), fresnel_refl_dielectric(eta, ac),
             fresnel_trans_dielectric(eta, ac), fresnel(c, ext, in), fresnel_schlick(eta, ac), schlick_weight(ac)});
    }
}

void refract_table(Rng& r, int n) {
    // wi n eta -> refract(wi, n, eta)
    std::printf("# refract 10\n");
    for (int k = 0; k < n; ++k) {
        Vec3f wi = unit(r), nn = unit(r);
        float eta = r.range(0.3f, 2.5f);
        Vec3f t = refract(wi, nn, eta);
        row({wi[0], wi[1], wi[2], nn[0], nn[1], nn[2], eta, t[0], t[1], t[2]});
    }
}

void frame_table(Rng& r, int n) {
    // n -> s t of Frame(n), and Frame(n).to_local(v) for a random v
    std::printf("# frame 15\n");
    for (int k = 0; k < n; ++k) {
        Vec3f nn = unit(r), v = unit(r);
        Frame fr(nn);
        Vec3f l = fr.to_local(v);
        row({nn[0], nn[1], nn[2], v[0], v[1], v[2], fr.s[0], fr.s[1], fr.s[2], fr.t[0], fr.t[1], fr.t[2], l[0], l[1],
             l[2]});
    }
}

void warp_table(Rng& r, int n) {
    // u1 u2 a b -> to_cosine_hemisphere(u) to_uniform_disk(u) sample_hemisphere(u) power_heuristic(1, a, 1, b)
    std::printf("# warps 13\n");
    for (int k = 0; k < n; ++k) {
        Vec2f u(r.uniform(), r.uniform());
        float a = r.range(0.f, 10.f), b = r.range(0.f, 10.f);
        Vec3f c = to_cosine_hemisphere(u);
        Vec2f d = to_uniform_disk(u);
        Vec3f h = sample_hemisphere(u);
        row({u[0], u[1], a, b, c[0], c[1], c[2], d[0], d[1], h[0], h[1], h[2], power_heuristic(1, a, 1, b)});
    }
}

}  // namespace

int main() {
    Rng r{20240611ull};
    mdf_table<GGXDist>("mdf_ggx", r, 1024);
    mdf_table<BeckmannDist>("mdf_beckmann", r, 1024);
    kpgloss_table(r, 2048);
    principle_specular_table(r, 1024);
    diffuse_table(r, 256);
    fresnel_table(r, 1024);
    refract_table(r, 512);
    frame_table(r, 512);
    warp_table(r, 512);
    return 0;
}
