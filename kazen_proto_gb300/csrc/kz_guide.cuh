// kz_guide.cuh — learned path guiding, device side: input encoding of a
// shading point, the 8-lobe von Mises-Fisher mixture the network predicts,
// its pdf, sampling, and the gradient of -log q with respect to the raw
// network outputs. Not part of the reference (kazen_proto has no guiding);
// the integrator MIS-combines this distribution with BSDF sampling so the
// estimator stays unbiased whatever the network predicts.
//
// Network: 51 inputs (position in the scene box, 3 axes x 8 frequency bands x
// {sin, cos} = 48, plus the geometric normal) -> 64 -> 64 -> 64 (ReLU) -> 40
// raw outputs = 8 lobes x (anchor point 3, concentration 1, weight 1); a
// lobe's mean direction points from the shading point to its anchor.
// vMF density (S. Jakob, "Numerically stable sampling of the von
// Mises-Fisher distribution on S^2", 2012):
//   v(w) = kappa / (2 pi (1 - exp(-2 kappa))) * exp(kappa (mu.w - 1)).
#pragma once

#include "kz_device.cuh"

namespace kz {

constexpr int kGuideIn = 51;
constexpr int kGuideInPad = 64;
constexpr int kGuideHidden = 64;
constexpr int kGuideLobes = 8;
constexpr int kGuideOut = 40;
constexpr int kGuideBands = 8;
constexpr float kKappaMin = 0.05f;
constexpr float kKappaMax = 2000.f;

// Parameter blob (FP32 master copy, and the BF16 copy the kernels read):
//   W1 [64][64] (out x in, inputs 51..63 zero), b1[64],
//   W2 [64][64], b2[64], W3 [64][64], b3[64], W4 [40][64], b4[40]
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + 64 * 64;
constexpr int kOffW2 = kOffB1 + 64;
constexpr int kOffB2 = kOffW2 + 64 * 64;
constexpr int kOffW3 = kOffB2 + 64;
constexpr int kOffB3 = kOffW3 + 64 * 64;
constexpr int kOffW4 = kOffB3 + 64;
constexpr int kOffB4 = kOffW4 + 40 * 64;
constexpr int kGuideParams = kOffB4 + 40;  // 15,080 (14,016 live weights, layer-1 padding, 232 biases)

// Input features of a shading point: position p01 in [0,1]^3 of the scene
// box, normal n. Feature j: for j < 48, axis a = j / 16, band b = (j % 16) / 2,
// sin for even j, cos for odd j, of 2^b * pi * p01[a]; 48..50 the normal.
__device__ __forceinline__ float guide_feature(int j, f3 p01, f3 n, float band_scale) {
    if (j < 48) {
        const int a = j >> 4;
        const int b = (j & 15) >> 1;
        const float x = comp(p01, a) * (float)(1 << b) * (kPi * band_scale);
        return (j & 1) ? cosf(x) : sinf(x);
    }
    if (j < 51) return comp(n, j - 48);
    return 0.f;
}

// sin and cos of 2^b * pi * bs * x (the input encoding of every guiding
// kernel). The argument is reduced exactly, t - 2 rint(t / 2) in [-1, 1],
// before the fast hardware sine and cosine, whose absolute error on
// [-pi, pi] (~2^-21) is far below the BF16 rounding the features then get.
__device__ __forceinline__ void band_sincos(float x, int b, float bs, float& sn, float& cs) {
    const float t = x * (float)(1 << b) * bs;
    const float r = t - 2.f * rintf(0.5f * t);
    __sincosf(kPi * r, &sn, &cs);
}

struct VmfMixture {
    f3 mu[kGuideLobes];
    float kappa[kGuideLobes];
    float w[kGuideLobes];   // lobe probabilities (softmax)
    float lc[kGuideLobes];  // shading form: log(w) + log norm(kappa) - kappa
};

__device__ __forceinline__ float softplus(float x) { return x > 20.f ? x : log1pf(expf(x)); }

// Lobe axis: from the shading point p01 to the lobe's anchor (raw outputs
// 0..2, both in scene-box coordinates), in world units (ext = box extent).
// A light seen through an aperture, or a bright patch, is then one fixed
// anchor for every shading point instead of a direction that turns with the
// position; a far anchor still acts as a fixed direction.
__device__ __forceinline__ f3 lobe_axis(const float* q, f3 p01, f3 ext) {
    return hmul(mk(q[0], q[1], q[2]) - p01, ext);
}

__device__ __forceinline__ void mixture_from_raw(const float* r, f3 p01, f3 ext, VmfMixture& m) {
    float mx = -1e30f;
    for (int k = 0; k < kGuideLobes; ++k) mx = fmaxf(mx, r[5 * k + 4]);
    float s = 0.f;
    for (int k = 0; k < kGuideLobes; ++k) {
        const float* q = r + 5 * k;
        const f3 a = lobe_axis(q, p01, ext);
        const float l = sqrtf(dot(a, a));
        m.mu[k] = l > 1e-12f ? mk(a.x / l, a.y / l, a.z / l) : mk(0.f, 0.f, 1.f);
        m.kappa[k] = fminf(kKappaMin + softplus(q[3]), kKappaMax);
        m.w[k] = expf(q[4] - mx);
        s += m.w[k];
    }
    for (int k = 0; k < kGuideLobes; ++k) m.w[k] /= s;
}

__device__ __forceinline__ float vmf_log_norm(float kappa) {
    // log(kappa / (2 pi (1 - exp(-2 kappa))))
    return logf(kappa) - logf(2.f * kPi) - log1pf(-expf(-2.f * kappa));
}

__device__ __forceinline__ float mixture_pdf(const VmfMixture& m, f3 w) {
    float p = 0.f;
    for (int k = 0; k < kGuideLobes; ++k)
        p += m.w[k] * expf(vmf_log_norm(m.kappa[k]) + m.kappa[k] * (dot(m.mu[k], w) - 1.f));
    return p;
}

// Shading form of the mixture: the same lobes with each lobe's weight and
// normalisation folded into one log factor, so a pdf evaluation is one
// exponential per lobe; uses the fast hardware exp/log (relative error near
// 2^-21, far below the network's own BF16 error). Sampling and the pdf both
// use this form, so the estimator's weights match the sampled density.
__device__ __forceinline__ void mixture_for_shading(const float* r, f3 p01, f3 ext, VmfMixture& m) {
    float mx = -1e30f;
    for (int k = 0; k < kGuideLobes; ++k) mx = fmaxf(mx, r[5 * k + 4]);
    float s = 0.f;
    for (int k = 0; k < kGuideLobes; ++k) {
        const float* q = r + 5 * k;
        const f3 a = lobe_axis(q, p01, ext);
        const float l2 = dot(a, a);
        const float il = l2 > 1e-24f ? rsqrtf(l2) : 0.f;
        m.mu[k] = il > 0.f ? mk(a.x * il, a.y * il, a.z * il) : mk(0.f, 0.f, 1.f);
        const float z = q[3];
        const float sp = z > 20.f ? z : __logf(1.f + __expf(z));
        m.kappa[k] = fminf(kKappaMin + sp, kKappaMax);
        m.w[k] = __expf(q[4] - mx);
        s += m.w[k];
    }
    const float is = 1.f / s;
    for (int k = 0; k < kGuideLobes; ++k) {
        m.w[k] *= is;
        const float kap = m.kappa[k];
        // log(kappa / (2 pi (1 - exp(-2 kappa))))
        const float ln = __logf(kap) - 1.8378770664093453f - __logf(1.f - __expf(-2.f * kap));
        m.lc[k] = __logf(fmaxf(m.w[k], 1e-30f)) + ln - kap;
    }
}

__device__ __forceinline__ float mixture_pdf_shading(const VmfMixture& m, f3 w) {
    float p = 0.f;
#pragma unroll
    for (int k = 0; k < kGuideLobes; ++k) p += __expf(m.lc[k] + m.kappa[k] * dot(m.mu[k], w));
    return p;
}

// Sample: lobe by weight (u0, rescaled), then the vMF by inversion of its
// cosine CDF, w = 1 + log(u + (1-u) exp(-2 kappa)) / kappa.
__device__ __forceinline__ f3 mixture_sample(const VmfMixture& m, float u0, float u1, float u2) {
    int k = kGuideLobes - 1;
    float acc = 0.f;
    for (int j = 0; j < kGuideLobes; ++j) {
        if (u0 < acc + m.w[j]) {
            k = j;
            break;
        }
        acc += m.w[j];
    }
    const float kap = m.kappa[k];
    const float cw = fminf(1.f, fmaxf(-1.f, 1.f + logf(u1 + (1.f - u1) * expf(-2.f * kap)) / kap));
    const float sw = sqrtf(fmaxf(0.f, 1.f - cw * cw));
    float sp, cp;
    sincosf(2.f * kPi * u2, &sp, &cp);
    const f3 n = m.mu[k];
    // orthonormal basis around mu (Duff et al., "Building an Orthonormal Basis, Revisited", JCGT 2017)
    const float sgn = copysignf(1.f, n.z);
    const float a = -1.f / (sgn + n.z);
    const float b = n.x * n.y * a;
    const f3 t = mk(1.f + sgn * n.x * n.x * a, sgn * b, -sgn * n.x);
    const f3 bb = mk(b, sgn + n.y * n.y * a, -n.y);
    return normalize(t * (sw * cp) + bb * (sw * sp) + n * cw);
}

// d(-log q(w)) / d(raw outputs), scaled by `scale`; returns -log q(w).
__device__ __forceinline__ float mixture_nll_grad(const float* r, f3 w, float scale, float* g, f3 p01, f3 ext) {
    VmfMixture m;
    mixture_from_raw(r, p01, ext, m);
    float v[kGuideLobes], dlogv_dk[kGuideLobes];
    float q = 0.f;
    for (int k = 0; k < kGuideLobes; ++k) {
        const float kap = m.kappa[k];
        const float e = expf(-2.f * kap);
        v[k] = expf(vmf_log_norm(kap) + kap * (dot(m.mu[k], w) - 1.f));
        dlogv_dk[k] = 1.f / kap - 2.f * e / (1.f - e) + (dot(m.mu[k], w) - 1.f);
        q += m.w[k] * v[k];
    }
    q = fmaxf(q, 1e-30f);
    for (int k = 0; k < kGuideLobes; ++k) {
        const float* rk = r + 5 * k;
        float* gk = g + 5 * k;
        const float resp = m.w[k] * v[k] / q;  // responsibility
        // softmax logit
        gk[4] = scale * (m.w[k] - resp);
        // concentration: kappa = kmin + softplus(z), clamped
        const float kap_raw = kKappaMin + softplus(rk[3]);
        const float dk_dz = kap_raw < kKappaMax ? 1.f / (1.f + expf(-rk[3])) : 0.f;
        gk[3] = scale * (-resp * dlogv_dk[k] * dk_dz);
        // mean direction: mu = a / |a|, a = (anchor - p01) * ext;
        // d log v / d mu = kappa w, d a / d anchor = diag(ext)
        const f3 ax = lobe_axis(rk, p01, ext);
        const float l = sqrtf(dot(ax, ax));
        if (l > 1e-12f) {
            const f3 mu = m.mu[k];
            const float c = dot(mu, w);
            const f3 proj = hmul((w - mu * c) * (1.f / l), ext);  // diag(ext) (I - mu mu^T) w / |a|
            const float s = -resp * m.kappa[k] * scale;
            gk[0] = s * proj.x;
            gk[1] = s * proj.y;
            gk[2] = s * proj.z;
        } else {
            gk[0] = gk[1] = gk[2] = 0.f;
        }
    }
    return -logf(q);
}

}  // namespace kz
