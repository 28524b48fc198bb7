// Per-texel forward render, loss, adjoint and Adam update of the flash-lit
// GGX/Cook-Torrance SVBRDF model.
//
// The model is the one of Microfacet.eval (src/microfacet.py:84-120 in
// tflsguoyu/svbrdf-diff-renderer). Rendered pixel (i, j) of every view depends only
// on texel (i, j), so one thread owns one texel: it decodes the 9 parameters once,
// loops over the views keeping every per-view term (v, l, h, D, F, G) in registers,
// and accumulates the adjoint into a handful of per-texel sums. Nothing per-view is
// ever written to memory except, in the forward-only kernel, the render itself.
//
// Texture layout is the reference's planar [9][H][W] FP32 (channels 0:3 diffuse,
// 3:5 normal xy, 5 roughness, 6:9 specular; src/microfacet.py:72-77); targets and
// renders are planar [V][3][H][W].
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace svb {

constexpr float kEps = 1e-6f;                  // Microfacet.eps (src/microfacet.py:14)
constexpr float kPi = 3.14159265358979323846f;  // np.pi as the FP32 scalar ATen uses
constexpr float kInvGamma = 1.0f / 2.2f;        // output encode exponent (src/microfacet.py:120)
constexpr int kMaxViews = 64;

enum LossKind : int {
  kLossMSE = 0,       // mean((render - target)^2)            (src/optimization.py:14,28-29)
  kLossLog1p = 1,     // mean((log1p(render) - log1p(target))^2)
  kLossLog1pPre = 2,  // as kLossLog1p, targets already hold log1p(target)
};

// One view: camera and light position in cm. `coloc` is 1 when the two are bitwise equal
// (the reference's flash captures, src/capture.py:70-71); the co-located branch uses
// l = v and h = v exactly, which is what FP64 evaluation of the reference formula gives.
struct __align__(16) View {
  float cx, cy, cz, coloc;
  float lx, ly, lz, pad;
};

// ---- fast transcendental helpers (single PTX instructions) ----
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// log1p(u) for u in [0, 1] (renders and targets): one lg2 of 1+u, about 1e-7 absolute.
__device__ __forceinline__ float log1p_fast(float u) { return lg2_approx(1.0f + u) * 0.69314718055994531f; }

// Decoded maps of one texel (tex2map, src/microfacet.py:72-79) plus the factors the
// adjoint needs to map map-space gradients back to the 9 parameters.
struct Maps {
  float d[3];     // diffuse  ((t+1)/2)^2.2
  float s[3];     // specular ((t+1)/2)^2.2
  float f1[3];    // d/pi * (1 - s)            (src/microfacet.py:102-103)
  float r;        // roughness ((t+1)/2)^2.2
  float alpha;    // r^2 (the reference passes roughness**2 to GGX and Smith)
  float a2;       // alpha^2                   (src/microfacet.py:30)
  float k;        // alpha*0.5 + eps            (src/microfacet.py:51)
  float n[3];     // unit normal               (src/microfacet.py:64-70)
};

// x = ((t+1)/2)^2.2 and dx/dt = 1.1 * ((t+1)/2)^1.2. A base of 0 gives 0 for both
// (lg2 -> -inf -> ex2 -> 0), matching pow's value and its ATen gradient at 0.
__device__ __forceinline__ float decode22(float t, float* dxdt) {
  const float base = (t + 1.0f) * 0.5f;
  const float lb = lg2_approx(base);
  if (dxdt) *dxdt = 1.1f * ex2_approx(1.2f * lb);
  return ex2_approx(2.2f * lb);
}

__device__ __forceinline__ void decode(const float t[9], Maps& m) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    m.d[c] = decode22(t[c], nullptr);
    m.s[c] = decode22(t[6 + c], nullptr);
    m.f1[c] = m.d[c] / kPi * (1.0f - m.s[c]);
  }
  m.r = decode22(t[5], nullptr);
  m.alpha = m.r * m.r;
  m.a2 = m.alpha * m.alpha;
  m.k = m.alpha * 0.5f + kEps;
  // reconstruct_normal: clamp xy, z = sqrt(1 - clamp(x^2+y^2, 0, 1-eps)), normalise
  const float nx = fminf(fmaxf(t[3], -1.0f), 1.0f);
  const float ny = fminf(fmaxf(t[4], -1.0f), 1.0f);
  const float sxy = fminf(fmaxf(nx * nx + ny * ny, 0.0f), 1.0f - kEps);
  const float nz = sqrtf(1.0f - sxy);
  const float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
  m.n[0] = nx * inv;
  m.n[1] = ny * inv;
  m.n[2] = nz * inv;
}

// Per-texel adjoint sums over views (all unscaled by the loss normaliser).
struct Adj {
  float gf1[3];   // d/d f1_c
  float gs[3];    // d/d s_c through F
  float ga2;      // d/d alpha^2 through D
  float gk;       // d/d k through G
  float gn[3];    // d/d unit normal
  float gp[3];    // d/d light power
};

__device__ __forceinline__ void adj_zero(Adj& a) {
#pragma unroll
  for (int c = 0; c < 3; ++c) { a.gf1[c] = 0.f; a.gs[c] = 0.f; a.gn[c] = 0.f; a.gp[c] = 0.f; }
  a.ga2 = 0.f;
  a.gk = 0.f;
}

// Texel position of src/microfacet.py:16-19 in FP32, same operation order.
__device__ __forceinline__ void texel_pos(int i, int j, int res_w, int res_h, float size, float& px, float& py) {
  px = (((float)j + 0.5f) / (float)res_w - 0.5f) * size;
  py = -((((float)i + 0.5f) / (float)res_h - 0.5f) * size);
}

enum Mode : int { kModeFwd = 0, kModeBwd = 1, kModeFused = 2 };

// One view of one texel. MODE:
//   kModeFwd   : writes the 3 rendered channels to out[c]; optional loss vs tgt.
//   kModeBwd   : reads dL/d render from gin[c] and accumulates the adjoint.
//   kModeFused : reads the target, accumulates the loss, then the adjoint.
// `io` holds 3 values: the target (fused), the incoming gradient (bwd) or the output (fwd).
template <int MODE, int LOSS, bool GRAD_POW, bool COLOC>
__device__ __forceinline__ void texel_view(const Maps& m, float px, float py, const View& vw,
                                           const float P[3], float io[3], float& loss, Adj& a) {
  // ---- geometry (get_dir, src/microfacet.py:60-62, 91-93) ----
  const float vx0 = vw.cx - px, vy0 = vw.cy - py, vz0 = vw.cz;
  const float qv = vx0 * vx0 + vy0 * vy0 + vz0 * vz0;
  const float iv = rsqrt_approx(qv);
  const float vx = vx0 * iv, vy = vy0 * iv, vz = vz0 * iv;
  float lx, ly, lz, inv_d2, hx, hy, hz;
  float nv_raw, nl_raw, nh_raw, vh;
  nv_raw = m.n[0] * vx + m.n[1] * vy + m.n[2] * vz;
  if (COLOC) {
    // l == v, h == normalize(2v) == v, v.h == 1
    lx = vx; ly = vy; lz = vz;
    hx = vx; hy = vy; hz = vz;
    inv_d2 = iv * iv;
    nl_raw = nv_raw;
    nh_raw = nv_raw;
    vh = 1.0f;
  } else {
    const float lx0 = vw.lx - px, ly0 = vw.ly - py, lz0 = vw.lz;
    const float d2 = lx0 * lx0 + ly0 * ly0 + lz0 * lz0;
    const float il = rsqrt_approx(d2);
    inv_d2 = il * il;
    lx = lx0 * il; ly = ly0 * il; lz = lz0 * il;
    const float hx0 = lx + vx, hy0 = ly + vy, hz0 = lz + vz;
    const float ih = rsqrt_approx(hx0 * hx0 + hy0 * hy0 + hz0 * hz0);
    hx = hx0 * ih; hy = hy0 * ih; hz = hz0 * ih;
    nl_raw = m.n[0] * lx + m.n[1] * ly + m.n[2] * lz;
    nh_raw = m.n[0] * hx + m.n[1] * hy + m.n[2] * hz;
    vh = fmaxf(vx * hx + vy * hy + vz * hz, 0.0f);
  }
  const float nv = fmaxf(nv_raw, 0.0f);
  const float nl = fmaxf(nl_raw, 0.0f);
  const float nh = fmaxf(nh_raw, 0.0f);

  // ---- GGX D (src/microfacet.py:28-32) ----
  // den = c2*a2 + (1 - c2). For unit n and h, 1 - (n.h)^2 = |n x h|^2; the cross product
  // has no cancellation near the highlight (n.h -> 1), where 1 - c2 in FP32 loses most
  // of its digits. Where the reference clamps n.h to 0, 1 - c2 is exactly 1.
  const float c2 = nh * nh;
  float s2 = 1.0f;
  if (nh_raw > 0.0f) {
    const float x0 = m.n[1] * hz - m.n[2] * hy;
    const float x1 = m.n[2] * hx - m.n[0] * hz;
    const float x2 = m.n[0] * hy - m.n[1] * hx;
    s2 = x0 * x0 + x1 * x1 + x2 * x2;
  }
  const float den = c2 * m.a2 + s2;
  const float E = kPi * (den * den) + kEps;
  const float rE = rcp_approx(E);
  const float D = m.a2 * rE;
  // ---- Smith G (src/microfacet.py:47-52) ----
  const float omk = 1.0f - m.k;
  const float Bv = nv * omk + m.k;
  const float rBv = rcp_approx(Bv);
  const float G1v = nv * rBv;
  float Bl, rBl, G1l;
  if (COLOC) { Bl = Bv; rBl = rBv; G1l = G1v; }
  else { Bl = nl * omk + m.k; rBl = rcp_approx(Bl); G1l = nl * rBl; }
  const float G = G1v * G1l;
  // ---- Fresnel, spherical-Gaussian Schlick (src/microfacet.py:43-45) ----
  // co-located: v.h = 1, so sphg = 2^(-5.55473 - 6.98316) is a constant
  const float sphg = COLOC ? 1.6815858e-4f : ex2_approx((-5.55473f * vh - 6.98316f) * vh);
  // ---- f2 = D F G / (4 nv nl + eps), img = P f nl / d^2 (src/microfacet.py:109-117) ----
  const float Q = 4.0f * nv * nl + kEps;
  const float rQ = rcp_approx(Q);
  const float DGQ = D * G * rQ;
  const float W = nl * inv_d2;

  float gDGQ = 0.f, gW = 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float F = m.s[c] + (1.0f - m.s[c]) * sphg;
    const float f = m.f1[c] + DGQ * F;
    const float PW = P[c] * W;
    const float img = f * PW;
    const float x = fminf(fmaxf(img, kEps), 1.0f);             // clamp(eps, 1)
    const float xp = ex2_approx(lg2_approx(x) * (kInvGamma - 1.0f));  // x^(1/2.2 - 1)
    const float out = x * xp;                                   // x^(1/2.2)
    float gout;
    if (MODE == kModeFwd) {
      if (LOSS >= 0) {
        float e;
        if (LOSS == kLossMSE) e = out - io[c];
        else if (LOSS == kLossLog1p) e = log1pf(out) - log1pf(io[c]);
        else e = log1pf(out) - io[c];
        loss += e * e;
      }
      io[c] = out;
      continue;
    } else if (MODE == kModeBwd) {
      gout = io[c];
    } else {
      float e;
      if (LOSS == kLossMSE) { e = out - io[c]; gout = e; }
      else {
        const float lo = log1p_fast(out);
        e = (LOSS == kLossLog1p) ? lo - log1p_fast(io[c]) : lo - io[c];
        gout = e * rcp_approx(1.0f + out);
      }
      loss += e * e;
    }
    // d out / d img = (1/2.2) x^(1/2.2-1) inside [eps, 1] (clamp passes its bounds)
    const float gimg = (img >= kEps && img <= 1.0f) ? gout * kInvGamma * xp : 0.0f;
    const float gf = gimg * PW;
    gW += gimg * (P[c] * f);
    if (GRAD_POW) a.gp[c] += gimg * f * W;
    a.gf1[c] += gf;
    gDGQ += gf * F;
    a.gs[c] += gf * DGQ * (1.0f - sphg);
  }
  if (MODE == kModeFwd) return;

  // ---- adjoint of the shared terms ----
  float gnl = gW * inv_d2;
  const float gD = gDGQ * G * rQ;
  const float gG = gDGQ * D * rQ;
  const float gQ = -gDGQ * DGQ * rQ;
  float gnv = gQ * 4.0f * nl;
  gnl += gQ * 4.0f * nv;
  const float gG1v = gG * G1l;
  const float gG1l = gG * G1v;
  gnv += gG1v * m.k * rBv * rBv;
  gnl += gG1l * m.k * rBl * rBl;
  a.gk -= gG1v * nv * (1.0f - nv) * rBv * rBv + gG1l * nl * (1.0f - nl) * rBl * rBl;
  const float t2 = D * rE * (2.0f * kPi) * den;
  a.ga2 += gD * (rE - t2 * c2);
  float gnh = -gD * t2 * (m.a2 - 1.0f) * 2.0f * nh;
  // clamp(min=0) of the dot products passes the gradient where the dot is >= 0
  if (COLOC) {
    const float gsum = (nv_raw >= 0.0f) ? (gnv + gnl + gnh) : 0.0f;
    a.gn[0] += gsum * vx; a.gn[1] += gsum * vy; a.gn[2] += gsum * vz;
  } else {
    gnv = (nv_raw >= 0.0f) ? gnv : 0.0f;
    gnl = (nl_raw >= 0.0f) ? gnl : 0.0f;
    gnh = (nh_raw >= 0.0f) ? gnh : 0.0f;
    a.gn[0] += gnv * vx + gnl * lx + gnh * hx;
    a.gn[1] += gnv * vy + gnl * ly + gnh * hy;
    a.gn[2] += gnv * vz + gnl * lz + gnh * hz;
  }
}

// Map the per-texel adjoint sums back to the 9 texture parameters (tex2map and
// reconstruct_normal reversed). `scale` is the loss normaliser's factor (2/N).
__device__ __forceinline__ void adj_to_params(const float t[9], const Maps& m, const Adj& a, float scale,
                                              float g[9]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float dd, ds;
    decode22(t[c], &dd);
    decode22(t[6 + c], &ds);
    const float gd = a.gf1[c] * (1.0f - m.s[c]) / kPi;
    const float gs = a.gs[c] - a.gf1[c] * m.d[c] / kPi;
    g[c] = gd * dd * scale;
    g[6 + c] = gs * ds * scale;
  }
  float dr;
  decode22(t[5], &dr);
  const float galpha = a.ga2 * 2.0f * m.alpha + a.gk * 0.5f;
  g[5] = galpha * 2.0f * m.r * dr * scale;
  // normal: n = mvec/|mvec|, mvec = (nx, ny, sqrt(1 - clamp(nx^2+ny^2, 0, 1-eps)))
  const float nx = fminf(fmaxf(t[3], -1.0f), 1.0f);
  const float ny = fminf(fmaxf(t[4], -1.0f), 1.0f);
  const float s = nx * nx + ny * ny;
  const float sxy = fminf(fmaxf(s, 0.0f), 1.0f - kEps);
  const float nz = sqrtf(1.0f - sxy);
  const float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
  const float ndg = m.n[0] * a.gn[0] + m.n[1] * a.gn[1] + m.n[2] * a.gn[2];
  const float gmx = (a.gn[0] - m.n[0] * ndg) * inv;
  const float gmy = (a.gn[1] - m.n[1] * ndg) * inv;
  const float gmz = (a.gn[2] - m.n[2] * ndg) * inv;
  const float gsxy = (s >= 0.0f && s <= 1.0f - kEps) ? (-0.5f * gmz / nz) : 0.0f;
  const float gnx = gmx + gsxy * 2.0f * nx;
  const float gny = gmy + gsxy * 2.0f * ny;
  g[3] = (t[3] >= -1.0f && t[3] <= 1.0f) ? gnx * scale : 0.0f;
  g[4] = (t[4] >= -1.0f && t[4] <= 1.0f) ? gny * scale : 0.0f;
}

// ---------------------------------------------------------------- co-located fast path
// Flash captures put the light at the camera (src/capture.py:70-71; data/random/render.json).
// Then l = h = v, v.h = 1 and the Fresnel term F_c = s_c + (1 - s_c) 2^(-12.53789) no
// longer depends on the view: the per-view work shrinks to one normalisation, D, G and the
// per-channel encode/loss. Gradients below omit the output encode's 1/2.2 factor, which
// the per-texel map-back applies once.
constexpr float kSphgColoc = 1.6815858e-4f;  // 2^(-5.55473 - 6.98316)
constexpr float kInvPi = 0.318309886183790671f;
constexpr float kLn2 = 0.69314718055994531f;

struct TexelC {
  float n0, n1, n2;  // unit normal
  float px, py;      // texel position (cm)
  float a2, k, omk;  // alpha^2, Smith k, 1 - k
  float f1[3];       // d/pi (1 - s)
  float F[3];        // s + (1 - s) sphg
};

struct AccC {
  float gf1[3];  // sum over views of dL/d f   (= dL/d f1)
  float gfd[3];  // sum over views of dL/d f * D G / Q   (-> dL/d F)
  float ga2, gk;
  float gn0, gn1, gn2;  // dL/d n, accumulated against the unnormalised view vector
  float gp[3];
  float loss;
};

// One co-located view of one texel. `cam` = (cx, cy, cz, -); tg = targets of this view.
// For the log1p losses the error is kept in log2 units (e = log2(1+out) - log2(1+target)):
// the caller scales the loss by ln2^2 and the gradient by ln2.
template <int LOSS, bool GRAD_POW>
__device__ __forceinline__ void coloc_view(const TexelC& t, float4 cam, float P0, float P1, float P2,
                                           const float tg[3], AccC& a) {
  const float vx = cam.x - t.px, vy = cam.y - t.py, vz = cam.z;
  const float q = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
  const float iv = rsqrt_approx(q);
  const float inv_d2 = iv * iv;
  const float nv_raw = fmaf(t.n0, vx, fmaf(t.n1, vy, t.n2 * vz)) * iv;
  const float nv = fmaxf(nv_raw, 0.0f);
  // 1 - (n.v)^2 as |n x v|^2 (no cancellation at the highlight); 1 where n.v is clamped
  const float x0 = fmaf(t.n1, vz, -t.n2 * vy);
  const float x1 = fmaf(t.n2, vx, -t.n0 * vz);
  const float x2 = fmaf(t.n0, vy, -t.n1 * vx);
  const float s2c = fmaf(x0, x0, fmaf(x1, x1, x2 * x2)) * inv_d2;
  const float s2 = nv_raw > 0.0f ? s2c : 1.0f;
  const float c2 = nv * nv;
  const float den = fmaf(c2, t.a2, s2);
  const float rE = rcp_approx(fmaf(kPi, den * den, kEps));
  const float D = t.a2 * rE;
  const float rB = rcp_approx(fmaf(nv, t.omk, t.k));
  const float G1 = nv * rB;
  const float G = G1 * G1;
  const float rQ = rcp_approx(fmaf(4.0f, c2, kEps));
  const float DGQ = D * G * rQ;
  const float W = nv * inv_d2;
  const float P[3] = {P0, P1, P2};
  float gDGQ = 0.f, gW = 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float f = fmaf(DGQ, t.F[c], t.f1[c]);
    const float PW = P[c] * W;
    const float img = f * PW;
    const float x = fminf(fmaxf(img, kEps), 1.0f);
    const float xp = ex2_approx(lg2_approx(x) * (kInvGamma - 1.0f));  // x^(1/2.2 - 1)
    const float out = x * xp;
    float e, gout;
    if (LOSS == kLossMSE) {
      e = out - tg[c];
      gout = e;
    } else {
      const float op1 = 1.0f + out;
      e = (LOSS == kLossLog1p) ? lg2_approx(op1) - lg2_approx(1.0f + tg[c])
                               : fmaf(-tg[c], 1.44269504088896341f, lg2_approx(op1));
      gout = e * rcp_approx(op1);
    }
    a.loss = fmaf(e, e, a.loss);
    const float gimg = (x == img) ? gout * xp : 0.0f;  // clamp(eps, 1) passes its range
    const float gf = gimg * PW;
    gW = fmaf(gimg, P[c] * f, gW);
    if (GRAD_POW) a.gp[c] = fmaf(gimg * f, W, a.gp[c]);
    a.gf1[c] += gf;
    gDGQ = fmaf(gf, t.F[c], gDGQ);
    a.gfd[c] = fmaf(gf, DGQ, a.gfd[c]);
  }
  const float tq = gDGQ * rQ;
  const float gD = tq * G;
  const float gG1 = 2.0f * tq * D * G1;  // G = G1^2
  const float rB2 = rB * rB;
  float gnv = fmaf(gG1 * t.k, rB2, fmaf(-tq * DGQ * 8.0f, nv, gW * inv_d2));
  a.gk = fmaf(-gG1 * nv * (1.0f - nv), rB2, a.gk);
  const float t2 = D * rE * (2.0f * kPi) * den;
  a.ga2 = fmaf(gD, fmaf(-t2, c2, rE), a.ga2);
  gnv = fmaf(-gD * t2 * (t.a2 - 1.0f) * 2.0f, nv, gnv);
  const float gs = nv_raw >= 0.0f ? gnv * iv : 0.0f;
  a.gn0 = fmaf(gs, vx, a.gn0);
  a.gn1 = fmaf(gs, vy, a.gn1);
  a.gn2 = fmaf(gs, vz, a.gn2);
}

// x = ((t+1)/2)^2.2 and its derivative 1.1 ((t+1)/2)^1.2 = 1.1 x / base (0 at base 0).
__device__ __forceinline__ float pow22(float base) { return ex2_approx(2.2f * lg2_approx(base)); }
__device__ __forceinline__ float dpow22(float x, float base) { return base > 0.0f ? 1.1f * x * rcp_approx(base) : 0.0f; }

// Per-texel constants of the co-located loop from parameters clamped to [-1, 1].
__device__ __forceinline__ void coloc_prepare(const float t9[9], float px, float py, TexelC& t) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float d = pow22((t9[c] + 1.0f) * 0.5f);
    const float sp = pow22((t9[6 + c] + 1.0f) * 0.5f);
    const float oms = 1.0f - sp;
    t.f1[c] = d * kInvPi * oms;
    t.F[c] = fmaf(oms, kSphgColoc, sp);
  }
  const float r = pow22((t9[5] + 1.0f) * 0.5f);
  const float alpha = r * r;
  t.a2 = alpha * alpha;
  t.k = fmaf(alpha, 0.5f, kEps);
  t.omk = 1.0f - t.k;
  const float nx = t9[3], ny = t9[4];
  const float sxy = fminf(fmaf(nx, nx, ny * ny), 1.0f - kEps);
  const float nz = sqrt_approx(1.0f - sxy);
  const float inv = rsqrt_approx(fmaf(nx, nx, fmaf(ny, ny, nz * nz)));
  t.n0 = nx * inv;
  t.n1 = ny * inv;
  t.n2 = nz * inv;
  t.px = px;
  t.py = py;
}

__device__ __forceinline__ void acc_zero(AccC& a) {
#pragma unroll
  for (int c = 0; c < 3; ++c) { a.gf1[c] = 0.f; a.gfd[c] = 0.f; a.gp[c] = 0.f; }
  a.ga2 = a.gk = a.gn0 = a.gn1 = a.gn2 = a.loss = 0.f;
}

// Map the co-located sums back to dL/dt (scaled by `scale`, the loss normaliser) and
// return the texel's squared error. The maps are re-derived from t9 rather than kept live
// through the view loop.
template <int LOSS, bool GRAD_POW>
__device__ __forceinline__ float coloc_finish(const float t9[9], const TexelC& t, const AccC& a, float scale,
                                              float g[9], float gp[3]) {
  const float unit = (LOSS == kLossMSE) ? 1.0f : kLn2;  // log1p errors were kept in log2 units
  const float sc = scale * kInvGamma * unit;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float bd = (t9[c] + 1.0f) * 0.5f, bs = (t9[6 + c] + 1.0f) * 0.5f;
    const float d = pow22(bd), sp = pow22(bs);
    g[c] = a.gf1[c] * (1.0f - sp) * kInvPi * dpow22(d, bd) * sc;
    g[6 + c] = fmaf(a.gfd[c], 1.0f - kSphgColoc, -a.gf1[c] * d * kInvPi) * dpow22(sp, bs) * sc;
  }
  const float br = (t9[5] + 1.0f) * 0.5f;
  const float r = pow22(br);
  const float alpha = r * r;
  const float galpha = fmaf(a.ga2, 2.0f * alpha, a.gk * 0.5f);
  g[5] = galpha * 2.0f * r * dpow22(r, br) * sc;
  // normal: n = m/|m|, m = (nx, ny, sqrt(1 - min(nx^2+ny^2, 1-eps)))
  const float nx = t9[3], ny = t9[4];
  const float sxy_raw = fmaf(nx, nx, ny * ny);
  const float nz = sqrt_approx(1.0f - fminf(sxy_raw, 1.0f - kEps));
  const float inv = rsqrt_approx(fmaf(nx, nx, fmaf(ny, ny, nz * nz)));
  const float ndg = t.n0 * a.gn0 + t.n1 * a.gn1 + t.n2 * a.gn2;
  const float gmx = (a.gn0 - t.n0 * ndg) * inv;
  const float gmy = (a.gn1 - t.n1 * ndg) * inv;
  const float gmz = (a.gn2 - t.n2 * ndg) * inv;
  const float gsxy = (sxy_raw <= 1.0f - kEps) ? (-0.5f * gmz * rcp_approx(nz)) : 0.0f;
  g[3] = fmaf(gsxy * 2.0f, nx, gmx) * sc;
  g[4] = fmaf(gsxy * 2.0f, ny, gmy) * sc;
  if (GRAD_POW) {
    gp[0] += a.gp[0] * sc;
    gp[1] += a.gp[1] * sc;
    gp[2] += a.gp[2] * sc;
  }
  return (LOSS == kLossMSE) ? a.loss : a.loss * (kLn2 * kLn2);
}

// Render, loss and adjoint of one texel whose views are all co-located. `t9` holds the
// parameters already clamped to [-1, 1]; targets come from tgt_at(v, tg[3]).
template <int LOSS, bool GRAD_POW, typename TgtFn>
__device__ __forceinline__ float coloc_texel(const float t9[9], float px, float py, int V, const View* views,
                                             const float P[3], float scale, TgtFn tgt_at, float g[9], float gp[3]) {
  TexelC t;
  coloc_prepare(t9, px, py, t);
  AccC a;
  acc_zero(a);
  const float P0 = P[0], P1 = P[1], P2 = P[2];
  for (int v = 0; v < V; ++v) {
    float tg[3];
    tgt_at(v, tg);
    const View& w = views[v];
    coloc_view<LOSS, GRAD_POW>(t, make_float4(w.cx, w.cy, w.cz, 0.f), P0, P1, P2, tg, a);
  }
  return coloc_finish<LOSS, GRAD_POW>(t9, t, a, scale, g, gp);
}

// ---------------------------------------------------------------- packed two-view path
// Blackwell issues FP32x2 (FFMA2/FMUL2/FADD2): one instruction does the same FP32 work
// on two lanes. The co-located loop runs two views per step, lane x = view v and lane
// y = view v+1, with the texel constants broadcast into both lanes; MUFU, min/max and
// select stay per lane.
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(rcp_approx(a.x), rcp_approx(a.y)); }
__device__ __forceinline__ float2 rsqrt2(float2 a) { return make_float2(rsqrt_approx(a.x), rsqrt_approx(a.y)); }
__device__ __forceinline__ float2 lg22(float2 a) { return make_float2(lg2_approx(a.x), lg2_approx(a.y)); }
__device__ __forceinline__ float2 ex22(float2 a) { return make_float2(ex2_approx(a.x), ex2_approx(a.y)); }

struct TexelC2 {
  float2 n0, n1, n2, mn0, mn1, mn2;  // unit normal and its negation
  float2 mpx, mpy;                   // -position
  float2 a2, k, omk, ma2m1x2;        // alpha^2, k, 1-k, -2(alpha^2 - 1)
  float2 f1[3], F[3];
};

struct AccC2 {
  float2 gf1[3], gfd[3];
  float2 ga2, gk, gn0, gn1, gn2, loss;
};

__device__ __forceinline__ void pack_texel(const TexelC& t, TexelC2& u) {
  u.n0 = bc2(t.n0); u.n1 = bc2(t.n1); u.n2 = bc2(t.n2);
  u.mn0 = bc2(-t.n0); u.mn1 = bc2(-t.n1); u.mn2 = bc2(-t.n2);
  u.mpx = bc2(-t.px); u.mpy = bc2(-t.py);
  u.a2 = bc2(t.a2); u.k = bc2(t.k); u.omk = bc2(t.omk); u.ma2m1x2 = bc2(-2.0f * (t.a2 - 1.0f));
#pragma unroll
  for (int c = 0; c < 3; ++c) { u.f1[c] = bc2(t.f1[c]); u.F[c] = bc2(t.F[c]); }
}

__device__ __forceinline__ void acc2_zero(AccC2& a) {
  const float2 z = make_float2(0.f, 0.f);
#pragma unroll
  for (int c = 0; c < 3; ++c) { a.gf1[c] = z; a.gfd[c] = z; }
  a.ga2 = a.gk = a.gn0 = a.gn1 = a.gn2 = a.loss = z;
}

// Fold the two lanes into the scalar accumulator.
__device__ __forceinline__ void acc2_fold(const AccC2& p, AccC& a) {
#pragma unroll
  for (int c = 0; c < 3; ++c) { a.gf1[c] += p.gf1[c].x + p.gf1[c].y; a.gfd[c] += p.gfd[c].x + p.gfd[c].y; }
  a.ga2 += p.ga2.x + p.ga2.y;
  a.gk += p.gk.x + p.gk.y;
  a.gn0 += p.gn0.x + p.gn0.y;
  a.gn1 += p.gn1.x + p.gn1.y;
  a.gn2 += p.gn2.x + p.gn2.y;
  a.loss += p.loss.x + p.loss.y;
}

// Views v (lane x) and v+1 (lane y) of one co-located texel: the arithmetic of coloc_view.
// cx/cy/cz are the two cameras, PP the light power broadcast, tg[c] the two targets. With
// LANE_X_ONLY the y lane is a placeholder (an odd view count's last view): its error is
// zeroed, so it adds nothing to the loss or the gradients.
template <int LOSS, bool LANE_X_ONLY = false>
__device__ __forceinline__ void coloc_view2(const TexelC2& t, float2 cx, float2 cy, float2 cz, const float2 PP[3],
                                            const float2 tg[3], AccC2& a) {
  const float2 vx = add2(cx, t.mpx), vy = add2(cy, t.mpy), vz = cz;
  const float2 q = fma2(vx, vx, fma2(vy, vy, mul2(vz, vz)));
  const float2 iv = rsqrt2(q);
  const float2 inv_d2 = mul2(iv, iv);
  const float2 nvr = mul2(fma2(t.n0, vx, fma2(t.n1, vy, mul2(t.n2, vz))), iv);
  const float2 nv = make_float2(fmaxf(nvr.x, 0.0f), fmaxf(nvr.y, 0.0f));
  const float2 x0 = fma2(t.n1, vz, mul2(t.mn2, vy));
  const float2 x1 = fma2(t.n2, vx, mul2(t.mn0, vz));
  const float2 x2 = fma2(t.n0, vy, mul2(t.mn1, vx));
  const float2 s2c = mul2(fma2(x0, x0, fma2(x1, x1, mul2(x2, x2))), inv_d2);
  const float2 s2 = make_float2(nvr.x > 0.0f ? s2c.x : 1.0f, nvr.y > 0.0f ? s2c.y : 1.0f);
  const float2 c2 = mul2(nv, nv);
  const float2 den = fma2(c2, t.a2, s2);
  const float2 rE = rcp2(fma2(bc2(kPi), mul2(den, den), bc2(kEps)));
  const float2 D = mul2(t.a2, rE);
  const float2 rB = rcp2(fma2(nv, t.omk, t.k));
  const float2 G1 = mul2(nv, rB);
  const float2 rQ = rcp2(fma2(bc2(4.0f), c2, bc2(kEps)));
  const float2 DGQ = mul2(mul2(D, mul2(G1, G1)), rQ);
  const float2 W = mul2(nv, inv_d2);
  float2 gDGQ = make_float2(0.f, 0.f), gW = make_float2(0.f, 0.f);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float2 f = fma2(DGQ, t.F[c], t.f1[c]);
    const float2 PW = mul2(PP[c], W);
    const float2 img = mul2(f, PW);
    const float2 x = make_float2(fminf(fmaxf(img.x, kEps), 1.0f), fminf(fmaxf(img.y, kEps), 1.0f));
    const float2 xp = ex22(mul2(lg22(x), bc2(kInvGamma - 1.0f)));
    const float2 out = mul2(x, xp);
    float2 e, gout;
    if (LOSS == kLossMSE) {
      e = add2(out, make_float2(-tg[c].x, -tg[c].y));
      gout = e;
    } else {
      const float2 op1 = add2(out, bc2(1.0f));
      const float2 lo = lg22(op1);
      e = (LOSS == kLossLog1p) ? add2(lo, make_float2(-lg2_approx(1.0f + tg[c].x), -lg2_approx(1.0f + tg[c].y)))
                               : fma2(tg[c], bc2(-1.44269504088896341f), lo);
      gout = mul2(e, rcp2(op1));
    }
    if (LANE_X_ONLY) {
      e.y = 0.0f;
      gout.y = 0.0f;
    }
    a.loss = fma2(e, e, a.loss);
    const float2 gm = mul2(gout, xp);
    const float2 gimg = make_float2(x.x == img.x ? gm.x : 0.0f, x.y == img.y ? gm.y : 0.0f);
    const float2 gf = mul2(gimg, PW);
    gW = fma2(gimg, mul2(PP[c], f), gW);
    a.gf1[c] = add2(a.gf1[c], gf);
    gDGQ = fma2(gf, t.F[c], gDGQ);
    a.gfd[c] = fma2(gf, DGQ, a.gfd[c]);
  }
  const float2 tq = mul2(gDGQ, rQ);
  const float2 gD = mul2(tq, mul2(G1, G1));
  const float2 gG1 = mul2(mul2(tq, D), add2(G1, G1));
  const float2 rB2 = mul2(rB, rB);
  float2 gnv = fma2(mul2(gG1, t.k), rB2, fma2(mul2(tq, mul2(DGQ, bc2(-8.0f))), nv, mul2(gW, inv_d2)));
  a.gk = fma2(mul2(mul2(gG1, nv), fma2(nv, bc2(1.0f), bc2(-1.0f))), rB2, a.gk);  // -gG1 nv (1-nv) rB^2
  const float2 t2 = mul2(mul2(D, rE), mul2(bc2(2.0f * kPi), den));
  a.ga2 = fma2(gD, fma2(mul2(t2, bc2(-1.0f)), c2, rE), a.ga2);
  gnv = fma2(mul2(mul2(gD, t2), t.ma2m1x2), nv, gnv);
  const float2 gsv = mul2(gnv, iv);
  const float2 gs = make_float2(nvr.x >= 0.0f ? gsv.x : 0.0f, nvr.y >= 0.0f ? gsv.y : 0.0f);
  a.gn0 = fma2(gs, vx, a.gn0);
  a.gn1 = fma2(gs, vy, a.gn1);
  a.gn2 = fma2(gs, vz, a.gn2);
}

// ---------------------------------------------------------------- texel-pair path
// Two adjacent texels per thread: lane x = texel i, lane y = texel i+1, one view at a time
// with the camera broadcast into both lanes. coloc_view2 is lane-generic, so it serves
// unchanged; the per-texel set-up and map-back below run on both texels at once, which
// the view-pair form has to do in scalar code.
__device__ __forceinline__ float2 clamp2(float2 t) {
  return make_float2(fminf(fmaxf(t.x, -1.0f), 1.0f), fminf(fmaxf(t.y, -1.0f), 1.0f));
}
__device__ __forceinline__ float2 half_up2(float2 t) { return fma2(t, bc2(0.5f), bc2(0.5f)); }  // (t+1)/2
__device__ __forceinline__ float2 one_minus2(float2 t) { return fma2(t, bc2(-1.0f), bc2(1.0f)); }
__device__ __forceinline__ float2 neg2(float2 t) { return make_float2(-t.x, -t.y); }

// pow22 of both lanes and, from the same lg2, d/dt = 1.1 base^1.2 (0 at base 0).
__device__ __forceinline__ float2 pow22_2(float2 base) { return ex22(mul2(bc2(2.2f), lg22(base))); }
__device__ __forceinline__ float2 pow22_2d(float2 base, float2& dxdt) {
  const float2 lb = lg22(base);
  dxdt = mul2(bc2(1.1f), ex22(mul2(bc2(1.2f), lb)));
  return ex22(mul2(bc2(2.2f), lb));
}

// Per-texel constants of two texels. The light power is folded in: Pf1[c] = P_c f1_c and
// PF[c] = P_c F_c, so a view computes P_c f_c = DGQ PF[c] + Pf1[c] with no P multiply.
struct TexelPair {
  float2 n0, n1, n2;  // unit normal
  float2 mpx, mpy;    // -position
  float2 a2, k, K1;   // alpha^2, Smith k, 4 pi (1 - alpha^2)
  float2 Pf1[3], PF[3];
};

// coloc_prepare for two texels. t9 = parameters already clamped to [-1, 1]; P = light power.
__device__ __forceinline__ void coloc_prepare_pair(const float2 t9[9], float2 px, float2 py, const float P[3],
                                                   TexelPair& u) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float2 d = pow22_2(half_up2(t9[c]));
    const float2 sp = pow22_2(half_up2(t9[6 + c]));
    const float2 oms = one_minus2(sp);
    u.Pf1[c] = mul2(mul2(mul2(d, bc2(kInvPi)), oms), bc2(P[c]));
    u.PF[c] = mul2(fma2(oms, bc2(kSphgColoc), sp), bc2(P[c]));
  }
  const float2 r = pow22_2(half_up2(t9[5]));
  const float2 alpha = mul2(r, r);
  u.a2 = mul2(alpha, alpha);
  u.k = fma2(alpha, bc2(0.5f), bc2(kEps));
  u.K1 = mul2(bc2(4.0f * kPi), one_minus2(u.a2));
  const float2 nx = t9[3], ny = t9[4];
  const float2 s = fma2(nx, nx, mul2(ny, ny));
  const float2 sxy = make_float2(fminf(s.x, 1.0f - kEps), fminf(s.y, 1.0f - kEps));
  const float2 oz = one_minus2(sxy);
  const float2 nz = make_float2(sqrt_approx(oz.x), sqrt_approx(oz.y));
  const float2 inv = rsqrt2(fma2(nx, nx, fma2(ny, ny, mul2(nz, nz))));
  u.n0 = mul2(nx, inv);
  u.n1 = mul2(ny, inv);
  u.n2 = mul2(nz, inv);
  u.mpx = neg2(px);
  u.mpy = neg2(py);
}

// One co-located view of two texels (lanes), the camera broadcast: the arithmetic of
// coloc_view with the light power folded into the texel constants. a.gf1 and a.gfd
// accumulate dL/df1 and dL/dF divided by P_c; coloc_finish_pair multiplies P_c back;
// a.gk accumulates -dL/dk. Back-facing views (n.v <= 0) need no selects beyond the clamp of
// n.v itself: their weight W = max(n.v, 0) / d^2 is 0, so the image is clamped to eps, its
// gradient is 0, and every term below is an exact 0 times a finite value (the reference's
// 1 - c2 = 1 there, which only reaches D, which only reaches the zero-weighted image).
// 1 - (n.v)^2 is |v - (n.v) n|^2 / |v|^2, the squared length of v's component across n:
// no cancellation at the highlight, as with the cross product of coloc_view.
template <int LOSS>
__device__ __forceinline__ void coloc_view_pair(const TexelPair& t, float2 cx, float2 cy, float2 cz,
                                                const float2 tg[3], AccC2& a) {
  const float2 vx = add2(cx, t.mpx), vy = add2(cy, t.mpy), vz = cz;
  const float2 q = fma2(vx, vx, fma2(vy, vy, mul2(vz, vz)));
  const float2 iv = rsqrt2(q);
  const float2 inv_d2 = mul2(iv, iv);
  const float2 dn = fma2(t.n0, vx, fma2(t.n1, vy, mul2(t.n2, vz)));  // n.v, |v| units
  const float2 nvr = mul2(dn, iv);
  const float2 nv = make_float2(fmaxf(nvr.x, 0.0f), fmaxf(nvr.y, 0.0f));  // clamp(min=0)
  const float2 mdn = mul2(dn, bc2(-1.0f));
  const float2 r0 = fma2(t.n0, mdn, vx), r1 = fma2(t.n1, mdn, vy), r2 = fma2(t.n2, mdn, vz);
  const float2 s2 = mul2(fma2(r0, r0, fma2(r1, r1, mul2(r2, r2))), inv_d2);
  const float2 c2 = mul2(nv, nv);
  const float2 den = fma2(c2, t.a2, s2);
  const float2 rE = rcp2(fma2(bc2(kPi), mul2(den, den), bc2(kEps)));
  const float2 D = mul2(t.a2, rE);
  const float2 omn = one_minus2(nv);
  const float2 rB = rcp2(fma2(t.k, omn, nv));  // 1 / (nv (1-k) + k)
  const float2 G1 = mul2(nv, rB);
  const float2 G = mul2(G1, G1);
  const float2 rQ = rcp2(fma2(bc2(4.0f), c2, bc2(kEps)));
  const float2 DGQ = mul2(mul2(D, G), rQ);
  const float2 W = mul2(nv, inv_d2);
  float2 gDGQ = make_float2(0.f, 0.f), gW = make_float2(0.f, 0.f);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float2 f = fma2(DGQ, t.PF[c], t.Pf1[c]);  // P_c (f1 + DGQ F)
    const float2 img = mul2(f, W);
    const float2 x = make_float2(fminf(fmaxf(img.x, kEps), 1.0f), fminf(fmaxf(img.y, kEps), 1.0f));
    const float2 xp = ex22(mul2(lg22(x), bc2(kInvGamma - 1.0f)));
    const float2 out = mul2(x, xp);
    float2 e, gout;
    if (LOSS == kLossMSE) {
      e = fma2(tg[c], bc2(-1.0f), out);
      gout = e;
    } else {
      const float2 op1 = add2(out, bc2(1.0f));
      const float2 lo = lg22(op1);
      e = (LOSS == kLossLog1p) ? add2(lo, make_float2(-lg2_approx(1.0f + tg[c].x), -lg2_approx(1.0f + tg[c].y)))
                               : fma2(tg[c], bc2(-1.44269504088896341f), lo);
      gout = mul2(e, rcp2(op1));
    }
    a.loss = fma2(e, e, a.loss);
    const float2 gm = mul2(gout, xp);
    const float2 gimg = make_float2(x.x == img.x ? gm.x : 0.0f, x.y == img.y ? gm.y : 0.0f);
    const float2 gw = mul2(gimg, W);  // dL/d f1_c / P_c
    gW = fma2(gimg, f, gW);
    a.gf1[c] = add2(a.gf1[c], gw);
    gDGQ = fma2(gw, t.PF[c], gDGQ);
    a.gfd[c] = fma2(gw, DGQ, a.gfd[c]);
  }
  const float2 tq = mul2(gDGQ, rQ);
  const float2 gD = mul2(tq, G);
  const float2 gG1 = mul2(mul2(tq, D), add2(G1, G1));
  const float2 rB2 = mul2(rB, rB);
  float2 gnv = fma2(mul2(gG1, t.k), rB2, fma2(mul2(tq, mul2(DGQ, bc2(-8.0f))), nv, mul2(gW, inv_d2)));
  a.gk = fma2(mul2(mul2(gG1, nv), omn), rB2, a.gk);  // -dL/dk: gG1 nv (1-nv) rB^2
  const float2 t2 = mul2(mul2(D, rE), den);          // dD/d den = -2 pi t2
  a.ga2 = fma2(gD, fma2(t2, mul2(c2, bc2(-2.0f * kPi)), rE), a.ga2);
  gnv = fma2(mul2(mul2(gD, t2), t.K1), nv, gnv);     // d den/d nv = 2 nv (alpha^2 - 1)
  const float2 gs = mul2(gnv, iv);                   // 0 for back-facing views
  a.gn0 = fma2(gs, vx, a.gn0);
  a.gn1 = fma2(gs, vy, a.gn1);
  a.gn2 = fma2(gs, vz, a.gn2);
}

// coloc_finish for two texels: dL/dt of both (scaled by `scale`) and their squared errors.
// The maps are re-derived from t9 (clamped parameters); the unit normal comes from u.
template <int LOSS>
__device__ __forceinline__ float2 coloc_finish_pair(const float2 t9[9], const TexelPair& u, const AccC2& a,
                                                    const float P[3], float scale, float2 g[9]) {
  const float unit = (LOSS == kLossMSE) ? 1.0f : kLn2;  // log1p errors were kept in log2 units
  const float sc1 = scale * kInvGamma * unit;
  const float2 sc = bc2(sc1);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float2 dd, ds;
    const float2 d = pow22_2d(half_up2(t9[c]), dd);
    const float2 sp = pow22_2d(half_up2(t9[6 + c]), ds);
    const float2 gf1 = mul2(a.gf1[c], bc2(P[c]));
    const float2 gfd = mul2(a.gfd[c], bc2(P[c]));
    g[c] = mul2(mul2(mul2(gf1, mul2(one_minus2(sp), bc2(kInvPi))), dd), sc);
    const float2 gsp = fma2(gfd, bc2(1.0f - kSphgColoc), mul2(gf1, mul2(d, bc2(-kInvPi))));
    g[6 + c] = mul2(mul2(gsp, ds), sc);
  }
  float2 dr;
  const float2 r = pow22_2d(half_up2(t9[5]), dr);
  const float2 alpha = mul2(r, r);
  const float2 galpha = fma2(a.ga2, add2(alpha, alpha), mul2(a.gk, bc2(-0.5f)));  // a.gk holds -dL/dk
  g[5] = mul2(mul2(mul2(galpha, add2(r, r)), dr), sc);
  // normal: n = m/|m|, m = (nx, ny, sqrt(1 - min(nx^2+ny^2, 1-eps)))
  const float2 nx = t9[3], ny = t9[4];
  const float2 s = fma2(nx, nx, mul2(ny, ny));
  const float2 oz = make_float2(1.0f - fminf(s.x, 1.0f - kEps), 1.0f - fminf(s.y, 1.0f - kEps));
  const float2 nz = make_float2(sqrt_approx(oz.x), sqrt_approx(oz.y));
  const float2 inv = rsqrt2(fma2(nx, nx, fma2(ny, ny, mul2(nz, nz))));
  const float2 mndg = mul2(fma2(u.n0, a.gn0, fma2(u.n1, a.gn1, mul2(u.n2, a.gn2))), bc2(-1.0f));
  const float2 gmx = mul2(fma2(u.n0, mndg, a.gn0), inv);
  const float2 gmy = mul2(fma2(u.n1, mndg, a.gn1), inv);
  const float2 gmz = mul2(fma2(u.n2, mndg, a.gn2), inv);
  const float2 hz = mul2(mul2(bc2(-1.0f), gmz), rcp2(nz));  // -gmz/nz = 2 dL/d sxy
  const float2 gsxy2 = make_float2(s.x <= 1.0f - kEps ? hz.x : 0.0f, s.y <= 1.0f - kEps ? hz.y : 0.0f);
  g[3] = mul2(fma2(gsxy2, nx, gmx), sc);
  g[4] = mul2(fma2(gsxy2, ny, gmy), sc);
  return (LOSS == kLossMSE) ? a.loss : mul2(a.loss, bc2(kLn2 * kLn2));
}

// dL/d(light power) of two co-located texels from the view-loop sums of coloc_view_pair,
// scaled like coloc_finish_pair's gradients. The render is P_c (f1_c + DGQ F_c) W per view,
// so dL/dP_c = f1_c sum(dL/dimg W) + F_c sum(dL/dimg W DGQ) = f1_c a.gf1_c + F_c a.gfd_c
// (a.gf1 and a.gfd hold those sums; src/microfacet.py:117 and src/svbrdf.py:48-50).
template <int LOSS>
__device__ __forceinline__ void coloc_light_grad_pair(const float2 t9[9], const AccC2& a, float scale, float2 gp[3]) {
  const float unit = (LOSS == kLossMSE) ? 1.0f : kLn2;
  const float2 sc = bc2(scale * kInvGamma * unit);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float2 d = pow22_2(half_up2(t9[c]));
    const float2 sp = pow22_2(half_up2(t9[6 + c]));
    const float2 oms = one_minus2(sp);
    const float2 f1 = mul2(mul2(d, bc2(kInvPi)), oms);
    const float2 F = fma2(oms, bc2(kSphgColoc), sp);
    gp[c] = mul2(fma2(F, a.gfd[c], mul2(f1, a.gf1[c])), sc);
  }
}

// torch.optim.Adam's update for one element (amsgrad off, no weight decay):
//   m.lerp_(g, 1-b1); v.mul_(b2).addcmul_(g, g, 1-b2);
//   p.addcdiv_(m, sqrt(v)/sqrt(bc2) + eps, -lr/bc1)
struct AdamScalars {
  float one_minus_b1, b2, one_minus_b2, inv_bc2_sqrt, eps, neg_step_size;
};

// Two elements of the Adam update in FP32x2 (same arithmetic as adam_update per lane).
__device__ __forceinline__ void adam_update2(float2& p, float2& mo, float2& vo, float2 g, const AdamScalars& s) {
  mo = fma2(bc2(s.one_minus_b1), fma2(mo, bc2(-1.0f), g), mo);  // fma(m, -1, g) = g - m exactly
  vo = fma2(bc2(s.one_minus_b2), mul2(g, g), mul2(vo, bc2(s.b2)));
  const float2 den = fma2(make_float2(sqrt_approx(vo.x), sqrt_approx(vo.y)), bc2(s.inv_bc2_sqrt), bc2(s.eps));
  p = fma2(bc2(s.neg_step_size), mul2(mo, rcp2(den)), p);
}

__device__ __forceinline__ void adam_update(float& p, float& mo, float& vo, float g, const AdamScalars& s) {
  mo = mo + s.one_minus_b1 * (g - mo);
  vo = vo * s.b2 + s.one_minus_b2 * (g * g);
  const float denom = sqrt_approx(vo) * s.inv_bc2_sqrt + s.eps;
  p = p + s.neg_step_size * __fdividef(mo, denom);
}

}  // namespace svb
