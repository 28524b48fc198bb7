// Novel-view rendering of a material under an environment map: the video frames of
// src/scripts.py:44-59, which the reference renders with Mitsuba 3 on the CPU
// (src/mitsubarender.py:7-105, `direct` integrator, 256 samples per pixel). The scene is the
// same: a 0.3-scaled rectangle turned by (Y angle, X -15 deg, Z -5 deg) in front of a 50-degree
// perspective camera at (0, 0, 1) looking at the origin, carrying the material as a normal
// map over a 0.5 / 0.5 blend of a GGX conductor (alpha = roughness map, reflectance =
// specular map) and a diffuse lobe (diffuse map), lit by a lat-long environment map.
//
// One thread per pixel runs all its samples. Per camera sample (direct illumination):
//   * a camera ray that misses the rectangle sees the environment;
//   * on the rectangle: one environment sample (importance-sampled by luminance x sin theta,
//     piecewise constant) and one BSDF sample (component picked with probability 1/2: GGX
//     visible normals (Heitz 2018) or a cosine lobe), combined with the power heuristic.
// The rectangle is the only object and planar, so nothing occludes a direction above it.
// Random numbers are a counter-based hash of (seed, pixel, sample, dimension), so a CPU
// restatement can draw exactly the same ones.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "svbrdf_common.cuh"

namespace svb {
namespace env {

constexpr float kPiF = 3.14159265358979323846f;

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V3 normalize(V3 a) { return mul(a, 1.0f / sqrtf(dot(a, a))); }

// Hash of Jarzynski and Olano, "Hash Functions for GPU Rendering" (JCGT 2020), PCG variant.
__device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
  const uint32_t state = v * 747796405u + 2891336453u;
  const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}
// Uniform in [0, 1) with 24 random bits (exact in FP32 and FP64).
__device__ __forceinline__ float rnd(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) {
  const uint32_t h = pcg_hash(pcg_hash(pcg_hash(seed ^ pixel) + sample) + dim);
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

// Scene constants computed on the host (see svbrdf_envmap_render).
struct Scene {
  float rot[9];      // rectangle rotation, row-major world <- local
  float scale;       // 0.3
  float tan_half;    // tan(fov / 2)
  float intensity;   // emitter scale
  int res, H, W, He, We, spp;
  uint32_t seed;
};

// Bilinear lookup of planar map channel c at texture coordinates (s, t) in [0, 1], texel
// centres at (k + 0.5) / n, wrapping.
__device__ __forceinline__ float tex_bilinear(const float* __restrict__ plane, int H, int W, float s, float t) {
  const float x = s * W - 0.5f, y = t * H - 0.5f;
  const float fx = floorf(x), fy = floorf(y);
  const float ax = x - fx, ay = y - fy;
  int x0 = (int)fx, y0 = (int)fy;
  int x1 = x0 + 1, y1 = y0 + 1;
  x0 = ((x0 % W) + W) % W; x1 = ((x1 % W) + W) % W;
  y0 = ((y0 % H) + H) % H; y1 = ((y1 % H) + H) % H;
  const float a = __ldg(plane + y0 * W + x0), b = __ldg(plane + y0 * W + x1);
  const float c = __ldg(plane + y1 * W + x0), d = __ldg(plane + y1 * W + x1);
  return (1.0f - ay) * ((1.0f - ax) * a + ax * b) + ay * ((1.0f - ax) * c + ax * d);
}

// Direction <-> lat-long coordinates: u = atan2(d.x, -d.z) / (2 pi) (wrapped to [0, 1)),
// v = acos(d.y) / pi.
__device__ __forceinline__ void dir_to_uv(V3 d, float& u, float& v) {
  u = atan2f(d.x, -d.z) * (0.5f / kPiF);
  if (u < 0.0f) u += 1.0f;
  v = acosf(fminf(fmaxf(d.y, -1.0f), 1.0f)) * (1.0f / kPiF);
}

// Environment radiance (piecewise constant per texel, times the emitter scale) and the
// solid-angle pdf of the importance sampler for direction d.
__device__ __forceinline__ V3 env_eval(const Scene& sc, const float* __restrict__ env,
                                       const float* __restrict__ row_pdf, const float* __restrict__ col_pdf, V3 d,
                                       float& pdf) {
  float u, v;
  dir_to_uv(d, u, v);
  const int j = min((int)(u * sc.We), sc.We - 1), i = min((int)(v * sc.He), sc.He - 1);
  const float* e = env + ((size_t)i * sc.We + j) * 3;
  const float st = sinf(v * kPiF);
  pdf = st > 0.0f ? __ldg(row_pdf + i) * __ldg(col_pdf + (size_t)i * sc.We + j) * (float)sc.He * (float)sc.We /
                        (2.0f * kPiF * kPiF * st)
                  : 0.0f;
  return mul(v3(__ldg(e), __ldg(e + 1), __ldg(e + 2)), sc.intensity);
}

// First k in [0, n) with cdf[k + 1] > u (cdf[0] = 0, cdf[n] = 1).
__device__ __forceinline__ int cdf_search(const float* __restrict__ cdf, int n, float u) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(cdf + mid + 1) > u) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// Local shading quantities of the blended BSDF.
struct Mat {
  V3 kd, ks;
  float alpha;
};

__device__ __forceinline__ float ggx_d(float cos_h, float a2) {
  const float t = cos_h * cos_h * (a2 - 1.0f) + 1.0f;
  return a2 / (kPiF * t * t);
}
__device__ __forceinline__ float smith_g1(V3 w, float a2) {
  const float c2 = w.z * w.z;
  const float t2 = fmaxf(1.0f - c2, 0.0f) / fmaxf(c2, 1e-20f);
  return 2.0f / (1.0f + sqrtf(1.0f + a2 * t2));
}

// f(wi, wo) cos(wo) of 0.5 conductor + 0.5 diffuse, and its sampling pdf, in the local frame
// (z = shading normal, wi toward the camera).
__device__ __forceinline__ V3 bsdf_eval(const Mat& m, V3 wi, V3 wo, float& pdf) {
  pdf = 0.0f;
  if (wi.z <= 0.0f || wo.z <= 0.0f) return v3(0.f, 0.f, 0.f);
  const float a2 = m.alpha * m.alpha;
  const V3 h = normalize(add(wi, wo));
  const float D = ggx_d(h.z, a2);
  const float g1i = smith_g1(wi, a2);
  const float G = g1i * smith_g1(wo, a2);
  const float spec = D * G / (4.0f * wi.z);  // conductor without Fresnel loss, times cos(wo)
  const float diff = wo.z * (1.0f / kPiF);
  pdf = 0.5f * (g1i * D / (4.0f * wi.z)) + 0.5f * diff;
  return v3(0.5f * (m.ks.x * spec + m.kd.x * diff), 0.5f * (m.ks.y * spec + m.kd.y * diff),
            0.5f * (m.ks.z * spec + m.kd.z * diff));
}

// GGX visible-normal sample (Heitz 2018, "Sampling the GGX Distribution of Visible Normals").
__device__ __forceinline__ V3 sample_vndf(V3 wi, float alpha, float u1, float u2) {
  const V3 vh = normalize(v3(alpha * wi.x, alpha * wi.y, wi.z));
  const float lensq = vh.x * vh.x + vh.y * vh.y;
  const V3 t1 = lensq > 0.0f ? mul(v3(-vh.y, vh.x, 0.0f), 1.0f / sqrtf(lensq)) : v3(1.0f, 0.0f, 0.0f);
  const V3 t2 = cross(vh, t1);
  const float r = sqrtf(u1), phi = 2.0f * kPiF * u2;
  const float p1 = r * cosf(phi);
  float p2 = r * sinf(phi);
  const float s = 0.5f * (1.0f + vh.z);
  p2 = (1.0f - s) * sqrtf(fmaxf(1.0f - p1 * p1, 0.0f)) + s * p2;
  const V3 nh = add(add(mul(t1, p1), mul(t2, p2)), mul(vh, sqrtf(fmaxf(1.0f - p1 * p1 - p2 * p2, 0.0f))));
  return normalize(v3(alpha * nh.x, alpha * nh.y, fmaxf(nh.z, 0.0f)));
}

__device__ __forceinline__ float power_heuristic(float a, float b) {
  const float a2 = a * a, b2 = b * b;
  return a2 + b2 > 0.0f ? a2 / (a2 + b2) : 0.0f;
}

// sRGB-encoded [0, 1] value to linear (the IEC 61966-2-1 curve).
__device__ __forceinline__ float srgb_to_linear(float c) {
  return c <= 0.04045f ? c * (1.0f / 12.92f) : powf((c + 0.055f) * (1.0f / 1.055f), 2.4f);
}

// Lanes per pixel: the pixel's camera samples are dealt round-robin to a group of kGroup
// adjacent lanes and their sums combined by shuffles, so a 256^2 frame runs 8 x 65536 threads
// (one thread per pixel left most of the GPU's warp slots empty).
constexpr int kGroup = 8;

__global__ void __launch_bounds__(128) envmap_render_kernel(Scene sc, const float* __restrict__ tex,
                                                            const float* __restrict__ env,
                                                            const float* __restrict__ row_cdf,
                                                            const float* __restrict__ row_pdf,
                                                            const float* __restrict__ col_cdf,
                                                            const float* __restrict__ col_pdf,
                                                            float* __restrict__ image) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int pix = gid / kGroup, part = gid % kGroup;
  const bool live = pix < sc.res * sc.res;  // every lane stays for the group's shuffles
  const int py = live ? pix / sc.res : 0, px = live ? pix - py * sc.res : 0;
  const V3 R0 = v3(sc.rot[0], sc.rot[3], sc.rot[6]);  // world images of the local x, y, z axes
  const V3 R1 = v3(sc.rot[1], sc.rot[4], sc.rot[7]);
  const V3 R2 = v3(sc.rot[2], sc.rot[5], sc.rot[8]);
  const V3 org = v3(0.0f, 0.0f, 1.0f);
  const size_t plane = (size_t)sc.H * sc.W;
  V3 acc = v3(0.f, 0.f, 0.f);
  for (int s = live ? part : sc.spp; s < sc.spp; s += kGroup) {
    const float jx = rnd(sc.seed, pix, s, 0), jy = rnd(sc.seed, pix, s, 1);
    const float sx = (2.0f * (px + jx) / sc.res - 1.0f) * sc.tan_half;
    const float sy = (1.0f - 2.0f * (py + jy) / sc.res) * sc.tan_half;
    const V3 d = normalize(v3(sx, sy, -1.0f));
    // the rectangle: plane through the origin with normal R2, |local x|, |local y| <= 1
    const float dn = dot(d, R2);
    float t = -1.0f;
    if (fabsf(dn) > 1e-8f) t = -dot(org, R2) / dn;
    bool hit = false;
    float lx = 0.f, ly = 0.f;
    if (t > 0.0f) {
      const V3 p = add(org, mul(d, t));
      lx = dot(p, R0) / sc.scale;
      ly = dot(p, R1) / sc.scale;
      hit = fabsf(lx) <= 1.0f && fabsf(ly) <= 1.0f && dn < 0.0f;
    }
    if (!hit) {
      float pdf;
      acc = add(acc, env_eval(sc, env, row_pdf, col_pdf, d, pdf));
      continue;
    }
    // texture coordinates: u = (x + 1) / 2, rows from the top (local y = +1)
    const float su = 0.5f * (lx + 1.0f), tv = 1.0f - 0.5f * (ly + 1.0f);
    float m9[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m9[c] = tex_bilinear(tex + c * plane, sc.H, sc.W, su, tv);
    Mat m;
    // stored parameters in [-1, 1] -> the [0, 1] values the reference's PNG maps hold
    m.kd = v3(srgb_to_linear(0.5f * (m9[0] + 1.0f)), srgb_to_linear(0.5f * (m9[1] + 1.0f)),
              srgb_to_linear(0.5f * (m9[2] + 1.0f)));
    m.ks = v3(srgb_to_linear(0.5f * (m9[6] + 1.0f)), srgb_to_linear(0.5f * (m9[7] + 1.0f)),
              srgb_to_linear(0.5f * (m9[8] + 1.0f)));
    m.alpha = fmaxf(srgb_to_linear(0.5f * (m9[5] + 1.0f)), 1e-3f);
    const float nx = m9[3], ny = m9[4];
    const float nz = sqrtf(fmaxf(1.0f - nx * nx - ny * ny, 0.0f));
    // shading frame: the tangent-space normal on (R0, R1, R2), tangent R0 made orthogonal
    const V3 n = normalize(add(add(mul(R0, nx), mul(R1, ny)), mul(R2, nz)));
    const V3 ts = normalize(sub(R0, mul(n, dot(n, R0))));
    const V3 tt = cross(n, ts);
    const V3 wiw = mul(d, -1.0f);
    const V3 wi = v3(dot(wiw, ts), dot(wiw, tt), dot(wiw, n));
    V3 L = v3(0.f, 0.f, 0.f);
    // environment sample
    {
      const float u1 = rnd(sc.seed, pix, s, 2), u2 = rnd(sc.seed, pix, s, 3);
      const int i = cdf_search(row_cdf, sc.He, u1);
      const float r0 = __ldg(row_cdf + i), r1 = __ldg(row_cdf + i + 1);
      const float dv = r1 > r0 ? (u1 - r0) / (r1 - r0) : 0.5f;
      const float* cc = col_cdf + (size_t)i * (sc.We + 1);
      const int j = cdf_search(cc, sc.We, u2);
      const float c0 = __ldg(cc + j), c1 = __ldg(cc + j + 1);
      const float du = c1 > c0 ? (u2 - c0) / (c1 - c0) : 0.5f;
      const float theta = kPiF * (i + dv) / sc.He, phi = 2.0f * kPiF * (j + du) / sc.We;
      const float st = sinf(theta);
      const V3 dl = v3(st * sinf(phi), cosf(theta), -st * cosf(phi));
      if (dot(dl, R2) > 0.0f) {
        float pdf_l;
        const V3 Le = env_eval(sc, env, row_pdf, col_pdf, dl, pdf_l);
        const V3 wo = v3(dot(dl, ts), dot(dl, tt), dot(dl, n));
        float pdf_b;
        const V3 f = bsdf_eval(m, wi, wo, pdf_b);
        if (pdf_l > 0.0f) {
          const float w = power_heuristic(pdf_l, pdf_b) / pdf_l;
          L = add(L, v3(f.x * Le.x * w, f.y * Le.y * w, f.z * Le.z * w));
        }
      }
    }
    // BSDF sample
    if (wi.z > 0.0f) {
      const float uc = rnd(sc.seed, pix, s, 4), u1 = rnd(sc.seed, pix, s, 5), u2 = rnd(sc.seed, pix, s, 6);
      V3 wo;
      if (uc < 0.5f) {
        const V3 h = sample_vndf(wi, m.alpha, u1, u2);
        wo = sub(mul(h, 2.0f * dot(wi, h)), wi);
      } else {
        const float r = sqrtf(u1), phi = 2.0f * kPiF * u2;
        wo = v3(r * cosf(phi), r * sinf(phi), sqrtf(fmaxf(1.0f - u1, 0.0f)));
      }
      float pdf_b;
      const V3 f = bsdf_eval(m, wi, wo, pdf_b);
      const V3 dw = add(add(mul(ts, wo.x), mul(tt, wo.y)), mul(n, wo.z));
      if (pdf_b > 0.0f && dot(dw, R2) > 0.0f) {
        float pdf_l;
        const V3 Le = env_eval(sc, env, row_pdf, col_pdf, dw, pdf_l);
        const float w = power_heuristic(pdf_b, pdf_l) / pdf_b;
        L = add(L, v3(f.x * Le.x * w, f.y * Le.y * w, f.z * Le.z * w));
      }
    }
    acc = add(acc, L);
  }
#pragma unroll
  for (int o = kGroup / 2; o > 0; o >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
  }
  if (!live || part != 0) return;
  const float inv = 1.0f / sc.spp;
  float* o = image + (size_t)pix * 3;
  const float rgb[3] = {acc.x * inv, acc.y * inv, acc.z * inv};
#pragma unroll
  for (int c = 0; c < 3; ++c) o[c] = powf(fminf(fmaxf(rgb[c], 0.0f), 1.0f), 1.0f / 2.2f);
}

}  // namespace env
}  // namespace svb

using namespace svb;

extern "C" {

int svbrdf_envmap_render(const float* textures, int h, int w, const float* env, int he, int we, const float* row_cdf,
                         const float* row_pdf, const float* col_cdf, const float* col_pdf, float* image, int res,
                         float angle_deg, float intensity, int spp, unsigned seed, void* stream) {
  if (!textures || !env || !row_cdf || !row_pdf || !col_cdf || !col_pdf || !image)
    return fail(SVBRDF_ERR_INVALID, "envmap: null pointer");
  if (h < 1 || w < 1 || he < 2 || we < 2 || res < 1 || spp < 1 || (long long)res * res * env::kGroup > (1LL << 30))
    return fail(SVBRDF_ERR_INVALID, "envmap: bad sizes");
  env::Scene sc;
  // rotation R = Ry(angle) Rx(-15) Rz(-5), applied to local points (Mitsuba's rotate order
  // in src/mitsubarender.py:17, degrees, right-handed)
  const double k = 3.14159265358979323846 / 180.0;
  const double a = angle_deg * k, b = -15.0 * k, c = -5.0 * k;
  const double ry[9] = {cos(a), 0, sin(a), 0, 1, 0, -sin(a), 0, cos(a)};
  const double rx[9] = {1, 0, 0, 0, cos(b), -sin(b), 0, sin(b), cos(b)};
  const double rz[9] = {cos(c), -sin(c), 0, sin(c), cos(c), 0, 0, 0, 1};
  double t[9], r[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      t[i * 3 + j] = 0;
      for (int q = 0; q < 3; ++q) t[i * 3 + j] += rx[i * 3 + q] * rz[q * 3 + j];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      r[i * 3 + j] = 0;
      for (int q = 0; q < 3; ++q) r[i * 3 + j] += ry[i * 3 + q] * t[q * 3 + j];
    }
  for (int i = 0; i < 9; ++i) sc.rot[i] = (float)r[i];
  sc.scale = 0.3f;
  sc.tan_half = (float)tan(25.0 * k);  // fov 50 degrees
  sc.intensity = intensity;
  sc.res = res;
  sc.H = h;
  sc.W = w;
  sc.He = he;
  sc.We = we;
  sc.spp = spp;
  sc.seed = seed;
  const long long n = (long long)res * res * env::kGroup;
  env::envmap_render_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      sc, textures, env, row_cdf, row_pdf, col_cdf, col_pdf, image);
  return check_launch("envmap_render_kernel");
}

}  // extern "C"
