// sph_render.cu -- headless screen-space fluid rendering of the particles,
// the CUDA form of the reference's GL pipeline (Graphics/render_particles.cpp
// ScreenSpaceSet, CurvatureFlow_Use / BilateralFilter_Use, ScreenSpaceRender
// and the shaders Gbuffer.vs/.fs, CurvatureFlow.fs, BilateralFilter.fs,
// ScreenSpaceRender.fs) into device buffers; no window and no graphics API.
//
// Passes of one frame (W x H pixels):
//   k_project     per particle: eye and clip coordinates (modelview and
//                 projection as GL column-major 4x4), clip test on the point
//                 centre, window position and depth, sprite size
//                 pointRadius * pointScale / |eye| (clamped to [1, 1024]);
//                 counts the sprite in each 16 x 16 pixel tile its square
//                 reaches
//   scan          per-tile list offsets
//   k_bin         the particle index into each such tile's list
//   segment sort  each tile's list by particle index (the GL draw order)
//   k_tile_resolve one block per tile, one thread per pixel, the tile's
//                 sprites in draw order: the covered test (centre in the
//                 sprite square, inside its disc, as Gbuffer.fs discards),
//                 the depth test (GL_LESS against the cleared 1.0) and the
//                 blend SRC_ALPHA / ONE_MINUS_SRC_ALPHA of the sprite
//                 thickness t = 0.02 exp(-d^2 / 6); counts the fragments
//   k_curvature   curvature-flow iterations (CurvatureFlow.fs) or
//   k_bilateral   bilateral iterations (BilateralFilter.fs), ping-pong
//   k_shade       ScreenSpaceRender.fs: normals from depth, Fresnel,
//                 Lambert, absorption by thickness, gamma
// and, in sph_render_foam, the foam overlay SetFoam draws over that frame:
//   k_foam_project  up to two foam sprites per particle (Foam.vs, Foam.gs)
//   k_foam_cover    per covered pixel, atomicMax of the sprite's draw key
//                   (depth test GL_ALWAYS, no blending: the last one wins)
//   k_foam_resolve  Foam.fs for the winning sprite: colour and frag depth
// Depth textures are sampled nearest with repeat wrap, as the reference's
// textures are set up (render_particles.cpp:126-190, no wrap mode given).
// The cube map and the scene behind the fluid are textures of the app; they
// are constant colours here (env, background).
#include <cstdint>
#include <cuda_runtime.h>

#include "pibiti_sph.h"
#include "sph_internal.h"
#include "sph_segsort.cuh"

namespace sph {
namespace {

constexpr int kRBlock = 256;
constexpr float kMaxSprite = 1024.f;

struct Mat4 {
  float m[16];  // column-major: m[c * 4 + r]
};

struct Proj {  // one particle's sprite
  float wx, wy, wz, size;  // size 0: not drawn
};

__device__ __forceinline__ float4 mul4(const Mat4& a, float x, float y, float z, float w) {
  const float* m = a.m;
  float4 r;
  r.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], x), __fmul_rn(m[4], y)), __fmul_rn(m[8], z)), __fmul_rn(m[12], w));
  r.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[1], x), __fmul_rn(m[5], y)), __fmul_rn(m[9], z)), __fmul_rn(m[13], w));
  r.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[2], x), __fmul_rn(m[6], y)), __fmul_rn(m[10], z)), __fmul_rn(m[14], w));
  r.w = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[3], x), __fmul_rn(m[7], y)), __fmul_rn(m[11], z)), __fmul_rn(m[15], w));
  return r;
}

// Point size of the sprite shaders, pointRadius * (pointScale / dist).  The
// reference binds those uniforms crossed (render_particles.cpp:274-275 with
// :791-792, and :326-328 with :819-820): pointRadius receives m_ParScale and
// pointScale m_ParRadius, so the product is rounded as scale * (radius / dist).
__device__ __forceinline__ float sprite_extent(float radius, float scale, float dist) {
  return __fmul_rn(scale, __fdiv_rn(radius, dist));
}

// Window coordinates of a clip-space point inside the clip volume.
__device__ __forceinline__ bool to_window(float4 c, int W, int H, float& wx, float& wy, float& wz) {
  if (!(c.w > 0.f) || fabsf(c.x) > c.w || fabsf(c.y) > c.w || fabsf(c.z) > c.w) return false;
  const float nx = __fdiv_rn(c.x, c.w), ny = __fdiv_rn(c.y, c.w), nz = __fdiv_rn(c.z, c.w);
  wx = __fmul_rn(__fadd_rn(nx, 1.f), __fmul_rn(0.5f, (float)W));
  wy = __fmul_rn(__fadd_rn(ny, 1.f), __fmul_rn(0.5f, (float)H));
  wz = __fmul_rn(__fadd_rn(nz, 1.f), 0.5f);
  return true;
}

__device__ __forceinline__ float norm3(float x, float y, float z) {
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
}

// The sprite of one particle (Gbuffer.vs): eye = MV (x, y, z, 1), clip =
// P eye, point size from |eye|; window coordinates by the viewport
// transform.  Points whose centre lies outside the clip volume are not drawn.
__device__ __forceinline__ Proj project(const Mat4& mv, const Mat4& pr, float4 p, int W, int H,
                                        float radius, float scale) {
  Proj o = {0.f, 0.f, 0.f, 0.f};
  const float4 e = mul4(mv, p.x, p.y, p.z, 1.f);
  const float4 c = mul4(pr, e.x, e.y, e.z, e.w);
  if (!to_window(c, W, H, o.wx, o.wy, o.wz)) return o;
  o.size = fminf(fmaxf(sprite_extent(radius, scale, norm3(e.x, e.y, e.z)), 1.f), kMaxSprite);
  return o;
}

// Pixel range a sprite's square covers (pixel centres px + 0.5 in
// [wx - size/2, wx + size/2)), clipped to the image.
__device__ __forceinline__ void sprite_box(const Proj& s, int W, int H, int& x0, int& x1, int& y0, int& y1) {
  const float h = __fmul_rn(0.5f, s.size);
  x0 = max((int)ceilf(__fsub_rn(__fsub_rn(s.wx, h), 0.5f)), 0);
  x1 = min((int)ceilf(__fsub_rn(__fadd_rn(s.wx, h), 0.5f)) - 1, W - 1);
  y0 = max((int)ceilf(__fsub_rn(__fsub_rn(s.wy, h), 0.5f)), 0);
  y1 = min((int)ceilf(__fsub_rn(__fadd_rn(s.wy, h), 0.5f)) - 1, H - 1);
}

// Gbuffer.fs at pixel (px, py) of a sprite: the point coordinate (origin
// upper left), the disc test, and the squared distance from the centre in
// point-coordinate units of 2.  Returns a negative value outside the disc.
__device__ __forceinline__ float sprite_mag(const Proj& s, int px, int py) {
  const float sx = __fadd_rn(0.5f, __fdiv_rn(__fsub_rn(__fadd_rn((float)px, 0.5f), s.wx), s.size));
  const float ty = __fsub_rn(0.5f, __fdiv_rn(__fsub_rn(__fadd_rn((float)py, 0.5f), s.wy), s.size));
  const float nx = __fsub_rn(__fmul_rn(sx, 2.f), 1.f), ny = __fadd_rn(__fmul_rn(ty, -2.f), 1.f);
  const float mag = __fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny));
  return mag > 1.f ? -1.f : mag;
}

constexpr int kTile = 16;                   // tile side in pixels
constexpr int kTilePixels = kTile * kTile;  // threads of k_tile_resolve

// Tiles the square of a drawn sprite reaches (false: no pixel of the image).
__device__ __forceinline__ bool tile_range(const Proj& s, int W, int H, int& tx0, int& tx1, int& ty0,
                                           int& ty1) {
  int x0, x1, y0, y1;
  sprite_box(s, W, H, x0, x1, y0, y1);
  if (x1 < x0 || y1 < y0) return false;
  tx0 = x0 / kTile;
  tx1 = x1 / kTile;
  ty0 = y0 / kTile;
  ty1 = y1 / kTile;
  return true;
}

// Sprites, per-tile sprite counts, and the number of (sprite, tile) pairs.
__global__ void k_project(const float4* __restrict__ pos, uint32_t n, Mat4 mv, Mat4 pr, int W, int H,
                          float radius, float scale, Proj* __restrict__ out, uint32_t* __restrict__ tcount,
                          int TX, unsigned long long* __restrict__ pairs) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t m = 0;
  if (i < n) {
    const Proj s = project(mv, pr, pos[i], W, H, radius, scale);
    out[i] = s;
    int tx0, tx1, ty0, ty1;
    if (s.size > 0.f && tile_range(s, W, H, tx0, tx1, ty0, ty1)) {
      for (int ty = ty0; ty <= ty1; ++ty)
        for (int tx = tx0; tx <= tx1; ++tx) atomicAdd(tcount + ty * TX + tx, 1u);
      m = (uint32_t)((tx1 - tx0 + 1) * (ty1 - ty0 + 1));
    }
  }
  const uint32_t wm = __reduce_add_sync(0xffffffffu, m);  // <= 32 x 66 x 66
  if ((threadIdx.x & 31) == 0 && wm) atomicAdd(pairs, (unsigned long long)wm);
}

// The particle index into the list of every tile its sprite reaches.
__global__ void k_bin(const Proj* __restrict__ sp, uint32_t n, int W, int H, int TX,
                      uint32_t* __restrict__ cursor, uint32_t* __restrict__ tlist) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Proj s = sp[i];
  int tx0, tx1, ty0, ty1;
  if (!(s.size > 0.f) || !tile_range(s, W, H, tx0, tx1, ty0, ty1)) return;
  for (int ty = ty0; ty <= ty1; ++ty)
    for (int tx = tx0; tx <= tx1; ++tx) tlist[atomicAdd(cursor + ty * TX + tx, 1u)] = i;
}

struct BoxedSprite {
  float wx, wy, wz, size;
  int x0, x1, y0, y1;  // sprite_box
};

// One block per tile, one thread per pixel: the tile's sprites (sorted by
// particle index) in chunks through shared memory; per pixel, in draw order,
// the covered test, the depth test and the blend.  Adds the covered
// fragments to *frags.
__global__ void __launch_bounds__(kTilePixels)
k_tile_resolve(const Proj* __restrict__ sp, const uint32_t* __restrict__ tlist,
               const uint32_t* __restrict__ toff, const uint32_t* __restrict__ tcount, int W, int H, int TX,
               float* __restrict__ depth, float* __restrict__ thick, unsigned long long* __restrict__ frags) {
  __shared__ BoxedSprite sb[kTilePixels];
  const uint32_t t = blockIdx.x;
  const int px = (int)(t % (uint32_t)TX) * kTile + (int)(threadIdx.x % kTile);
  const int py = (int)(t / (uint32_t)TX) * kTile + (int)(threadIdx.x / kTile);
  const bool valid = px < W && py < H;
  const uint32_t s0 = toff[t], n = tcount[t];
  float d = 1.f, th = 0.f;
  uint32_t covered = 0;
  for (uint32_t c0 = 0; c0 < n; c0 += kTilePixels) {
    const uint32_t m = min(n - c0, (uint32_t)kTilePixels);
    __syncthreads();  // the previous chunk is consumed
    if (threadIdx.x < m) {
      const Proj s = sp[tlist[s0 + c0 + threadIdx.x]];
      BoxedSprite b = {s.wx, s.wy, s.wz, s.size, 0, -1, 0, -1};
      sprite_box(s, W, H, b.x0, b.x1, b.y0, b.y1);
      sb[threadIdx.x] = b;
    }
    __syncthreads();
    if (!valid) continue;
    for (uint32_t k = 0; k < m; ++k) {
      const BoxedSprite b = sb[k];
      if (px < b.x0 || px > b.x1 || py < b.y0 || py > b.y1) continue;
      const Proj s = {b.wx, b.wy, b.wz, b.size};
      const float mag = sprite_mag(s, px, py);
      if (mag < 0.f) continue;
      ++covered;
      if (s.wz < d) {
        const float tv = __fmul_rn(0.02f, expf(__fdiv_rn(-mag, 6.f)));
        d = s.wz;
        th = __fadd_rn(__fmul_rn(tv, tv), __fmul_rn(th, __fsub_rn(1.f, tv)));
      }
    }
  }
  if (valid) {
    depth[(size_t)py * W + px] = d;
    thick[(size_t)py * W + px] = th;
  }
  unsigned long long c = covered;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(frags, c);
}

// Foam overlay: Foam.vs, Foam.gs and Foam.fs as SetFoam draws them over the
// shaded frame (render_particles.cpp:306-334).  The shader's foam value w is
// the x of the attribute at location 3, which NVIDIA's GL driver aliases to
// the colour array _drawPoints binds (the step's colour output).  The
// geometry shader emits copy k of a point at gl_Position - k for each
// k < w (max_vertices = 2, so two copies at most), both with the particle's
// eye position and size.  Blending is off and the depth function is
// GL_ALWAYS, so every pixel keeps the last fragment in draw order (particle,
// then copy): the largest draw key that covers it.
struct FoamSprite {
  float wx, wy, size, w;  // window position, point size (0: not drawn), foam value
  float ex, ey, ez, r;    // eyeSpacePos.xyz, eyeSpaceRadius (unclamped)
};
constexpr float kFoamThreshold = 0.05f;

__global__ void k_foam_project(const float4* __restrict__ pos, const float4* __restrict__ clr, uint32_t n,
                               Mat4 mv, Mat4 pr, int W, int H, float radius, float scale,
                               FoamSprite* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i];
  const float w = clr[i].x;
  const float4 e = mul4(mv, p.x, p.y, p.z, p.w);  // ModelView * vPosition (the particle's own w)
  const float4 q = mul4(mv, p.x, p.y, p.z, 1.f);  // posEye
  const float r = sprite_extent(radius, scale, norm3(q.x, q.y, q.z));
  const float4 c = mul4(pr, e.x, e.y, e.z, e.w);
  for (int k = 0; k < 2; ++k) {
    FoamSprite s = {0.f, 0.f, 0.f, w, e.x, e.y, e.z, r};
    const float fk = -(float)k;  // gl_Position + vec4(-i)
    float wz;
    if ((float)k < w &&
        to_window(make_float4(__fadd_rn(c.x, fk), __fadd_rn(c.y, fk), __fadd_rn(c.z, fk), __fadd_rn(c.w, fk)),
                  W, H, s.wx, s.wy, wz))
      s.size = fminf(fmaxf(r, 1.f), kMaxSprite);
    out[2 * (size_t)i + k] = s;
  }
}

// Foam.fs at pixel (px, py): the point coordinate's offset from the centre
// scaled to [-1, 1] (nx, ny; origin upper left), its length d, and whether
// the fragment survives the discard d > clamp(w / 0.05, 0, 1).
__device__ __forceinline__ bool foam_frag(const FoamSprite& s, int px, int py, float& nx, float& ny, float& d) {
  const float sx = __fadd_rn(0.5f, __fdiv_rn(__fsub_rn(__fadd_rn((float)px, 0.5f), s.wx), s.size));
  const float ty = __fsub_rn(0.5f, __fdiv_rn(__fsub_rn(__fadd_rn((float)py, 0.5f), s.wy), s.size));
  nx = __fmul_rn(__fsub_rn(sx, 0.5f), 2.f);
  ny = __fmul_rn(__fsub_rn(ty, 0.5f), 2.f);
  d = __fsqrt_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)));
  return !(d > fminf(fmaxf(__fdiv_rn(s.w, kFoamThreshold), 0.f), 1.f));
}

// Per foam fragment: the pixel's draw key becomes the largest (sprite index + 1).
__global__ void k_foam_cover(const FoamSprite* __restrict__ sp, uint32_t m, int W, int H,
                             uint32_t* __restrict__ key) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const FoamSprite s = sp[j];
  if (!(s.size > 0.f)) return;
  const Proj b = {s.wx, s.wy, 0.f, s.size};
  int x0, x1, y0, y1;
  sprite_box(b, W, H, x0, x1, y0, y1);
  float nx, ny, d;
  for (int py = y0; py <= y1; ++py)
    for (int px = x0; px <= x1; ++px)
      if (foam_frag(s, px, py, nx, ny, d)) atomicMax(key + (size_t)py * W + px, j + 1);
}

// The winning fragment of each pixel: colour (1, 1, 1, alpha) over the frame
// and gl_FragDepth (the sphere point's linearised depth, near 0.1 and far
// 1000 as Foam.fs fixes them), clamped to [0, 1] as the depth buffer stores it.
__global__ void k_foam_resolve(const FoamSprite* __restrict__ sp, const uint32_t* __restrict__ key, int W,
                               int H, Mat4 pr, float4* __restrict__ rgba, float* __restrict__ fdepth) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (uint32_t)(W * H)) return;
  const uint32_t k = key[p];
  if (k == 0) {
    if (fdepth) fdepth[p] = 1.f;
    return;
  }
  const FoamSprite s = sp[k - 1];
  float nx, ny, d;
  foam_frag(s, (int)(p % (uint32_t)W), (int)(p / (uint32_t)W), nx, ny, d);
  const float nz = __fsqrt_rn(__fsub_rn(1.f, d));  // normal.z = sqrt(1 - dist), as written
  const float l = norm3(nx, -ny, nz);
  const float ux = __fdiv_rn(nx, l), uy = __fdiv_rn(-ny, l), uz = __fdiv_rn(nz, l);
  const float fh = (float)H;
  const float fx = __fadd_rn(s.ex, __fdiv_rn(__fmul_rn(ux, s.r), fh));
  const float fy = __fadd_rn(s.ey, __fdiv_rn(__fmul_rn(uy, s.r), fh));
  const float fz = __fadd_rn(s.ez, __fdiv_rn(__fmul_rn(uz, s.r), fh));
  const float4 c = mul4(pr, fx, fy, fz, 1.f);
  const float dd = __fdiv_rn(c.z, c.w);
  const float nearp = 0.1f, farp = 1000.f;
  const float fd = __fdiv_rn(__fmul_rn(2.f, nearp),
                             __fsub_rn(__fadd_rn(farp, nearp),
                                       __fmul_rn(__fadd_rn(__fmul_rn(dd, 0.5f), 0.5f), __fsub_rn(farp, nearp))));
  const float f = fminf(fmaxf(__fdiv_rn(s.w, kFoamThreshold), 0.f), 1.f);
  const float a = s.w >= kFoamThreshold ? 1.f : __fsub_rn(1.f, f);
  if (rgba) rgba[p] = make_float4(1.f, 1.f, 1.f, a);
  if (fdepth) fdepth[p] = fminf(fmaxf(fd, 0.f), 1.f);
}

// Nearest texel with repeat wrap.
__device__ __forceinline__ float tex(const float* __restrict__ z, int x, int y, int W, int H) {
  x %= W;
  if (x < 0) x += W;
  y %= H;
  if (y < 0) y += H;
  return z[(size_t)y * W + x];
}

struct Deriv {
  float dzx, dzy, dzx2, dzy2;
};

// dzdx / dzdy of the shaders (half central differences of neighbouring
// texels) and their second differences.
__device__ __forceinline__ Deriv derivs(const float* __restrict__ z, int x, int y, int W, int H) {
  auto dx = [&](int n) { return __fdiv_rn(__fsub_rn(tex(z, x + 1 + n, y, W, H), tex(z, x - 1 + n, y, W, H)), 2.f); };
  auto dy = [&](int n) { return __fdiv_rn(__fsub_rn(tex(z, x, y + 1 + n, W, H), tex(z, x, y - 1 + n, W, H)), 2.f); };
  Deriv r;
  r.dzx = dx(0);
  r.dzx2 = __fdiv_rn(__fsub_rn(dx(1), dx(-1)), 2.f);
  r.dzy = dy(0);
  r.dzy2 = __fdiv_rn(__fsub_rn(dy(1), dy(-1)), 2.f);
  return r;
}

// CurvatureFlow.fs: one iteration; texels with Z <= 0 or Z == 1 are
// discarded and keep the cleared 1.0.
__global__ void k_curvature(const float* __restrict__ zin, float* __restrict__ zout, int W, int H) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (uint32_t)(W * H)) return;
  const int x = (int)(p % (uint32_t)W), y = (int)(p / (uint32_t)W);
  const float Z = zin[p];
  if (Z <= 0.f || Z == 1.f) {
    zout[p] = 1.f;
    return;
  }
  const float i = __fdiv_rn(__fadd_rn((float)x, 0.5f), (float)W), j = __fdiv_rn(__fadd_rn((float)y, 0.5f), (float)H);
  const Deriv d = derivs(zin, x, y, W, H);
  const float Cx = __fdiv_rn(2.f, __fmul_rn((float)W, i)), Cy = __fdiv_rn(2.f, __fmul_rn((float)H, j));
  const float D = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(Cy, Cy), d.dzx), d.dzx),
                                      __fmul_rn(__fmul_rn(__fmul_rn(Cx, Cx), d.dzy), d.dzy)),
                            __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(Cx, Cx), Cy), Cy), Z), Z));
  const float inv_D32 = __fdiv_rn(1.f, powf(D, 1.5f));
  const float ky = __fdiv_rn(__fdiv_rn(4.f, (float)H), (float)H), kx = __fdiv_rn(__fdiv_rn(4.f, (float)W), (float)W);
  const float ii2 = powf(i, -2.f), ii3 = powf(i, -3.f), jj2 = powf(j, -2.f), jj3 = powf(j, -3.f);
  const float dDx = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(ky, jj2), 2.f), d.dzx), d.dzx2),
                                        __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(kx, d.dzy), d.dzy), -2.f), ii3)),
                              __fmul_rn(__fmul_rn(__fmul_rn(ky, jj2), kx),
                                        __fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(-2.f, ii3), Z), Z),
                                                  __fmul_rn(__fmul_rn(__fmul_rn(ii2, 2.f), Z), d.dzx))));
  const float dDy = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(kx, ii2), 2.f), d.dzy), d.dzy2),
                                        __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(ky, d.dzx), d.dzx), -2.f), jj3)),
                              __fmul_rn(__fmul_rn(__fmul_rn(kx, ii2), ky),
                                        __fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(-2.f, jj3), Z), Z),
                                                  __fmul_rn(__fmul_rn(__fmul_rn(jj2, 2.f), Z), d.dzy))));
  const float Ex = __fsub_rn(__fmul_rn(__fmul_rn(0.5f, d.dzx), dDx), __fmul_rn(d.dzx2, D));
  const float Ey = __fsub_rn(__fmul_rn(__fmul_rn(0.5f, d.dzy), dDy), __fmul_rn(d.dzy2, D));
  float flow = __fdiv_rn(__fmul_rn(__fadd_rn(__fmul_rn(Cy, Ex), __fmul_rn(Cx, Ey)), inv_D32), 2.f);
  if (flow > 1.f) flow = 1.f;
  if (flow < -1.f) flow = -1.f;
  float z = __fsub_rn(Z, __fmul_rn(flow, 0.001f));
  if (z > 1.f) z = 1.f;
  if (z < 0.f) z = 0.f;
  zout[p] = z;
}

__device__ __forceinline__ float normpdf(float x, float sigma) {
  return __fdiv_rn(__fmul_rn(0.39894f, expf(__fdiv_rn(__fmul_rn(__fmul_rn(-0.5f, x), x), __fmul_rn(sigma, sigma)))), sigma);
}

// BilateralFilter.fs: one iteration.  Its sample offset (i / W, j) / H moves
// less than one texel in x for |i| < H / 2, so with nearest sampling every
// i reads column x and the filter acts along y.
__global__ void k_bilateral(const float* __restrict__ zin, float* __restrict__ zout, int W, int H,
                            const float* __restrict__ kern, int kc, float sigma) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (uint32_t)(W * H)) return;
  const int x = (int)(p % (uint32_t)W), y = (int)(p / (uint32_t)W);
  const float Z = zin[p];
  if (Z == 0.f || Z == 1.f) {
    zout[p] = 1.f;
    return;
  }
  const float bZ = __fdiv_rn(1.f, normpdf(0.f, sigma));
  float num = 0.f, den = 0.f;
  for (int a = -kc; a <= kc; ++a)
    for (int b = -kc; b <= kc; ++b) {
      const float cv = tex(zin, x, y + b, W, H);
      const float f = __fmul_rn(__fmul_rn(__fmul_rn(normpdf(__fsub_rn(cv, Z), sigma), bZ), kern[kc + a]), kern[kc + b]);
      den = __fadd_rn(den, f);
      num = __fadd_rn(num, __fmul_rn(f, cv));
    }
  zout[p] = __fdiv_rn(num, den);
}

struct Shade {
  Mat4 mv_inv;  // inverse(ModelView)
  float p00, p11;
  float env[3], bg[3];
};

__device__ __forceinline__ float3 nrm(float3 v) {
  const float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y)), __fmul_rn(v.z, v.z)));
  return make_float3(__fdiv_rn(v.x, l), __fdiv_rn(v.y, l), __fdiv_rn(v.z, l));
}
__device__ __forceinline__ float dot3f(float3 a, float3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

// fresnel() of ScreenSpaceRender.fs.
__device__ __forceinline__ float fresnel(float rr1, float rr2, float3 n, float3 d) {
  const float r = __fdiv_rn(rr1, rr2);
  const float t1 = dot3f(n, make_float3(-d.x, -d.y, -d.z));
  const float t2 = __fsqrt_rn(__fsub_rn(1.f, __fmul_rn(__fmul_rn(r, r), __fsub_rn(1.f, __fmul_rn(t1, t1)))));
  float rs = __fdiv_rn(__fsub_rn(__fmul_rn(rr1, t1), __fmul_rn(rr2, t2)), __fadd_rn(__fmul_rn(rr1, t1), __fmul_rn(rr2, t2)));
  rs = __fmul_rn(rs, rs);
  float rp = __fdiv_rn(__fsub_rn(__fmul_rn(rr1, t2), __fmul_rn(rr2, t1)), __fadd_rn(__fmul_rn(rr1, t2), __fmul_rn(rr2, t1)));
  rp = __fmul_rn(rp, rp);
  return __fdiv_rn(__fadd_rn(rs, rp), 2.f);
}

__global__ void k_shade(const float* __restrict__ zin, const float* __restrict__ thick, int W, int H,
                        Shade sh, float4* __restrict__ rgba) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (uint32_t)(W * H)) return;
  const int x = (int)(p % (uint32_t)W), y = (int)(p / (uint32_t)W);
  const float4 bgc = make_float4(sh.bg[0], sh.bg[1], sh.bg[2], 1.f);
  const float Z = zin[p];
  if (Z <= 0.f || Z == 1.f) {
    rgba[p] = bgc;
    return;
  }
  const float gamma = 2.2f;
  const float thickness = __fmul_rn(thick[p], 0.075f);
  const float i = __fdiv_rn(__fadd_rn((float)x, 0.5f), (float)W), j = __fdiv_rn(__fadd_rn((float)y, 0.5f), (float)H);
  // getNormals
  const Deriv d = derivs(zin, x, y, W, H);
  const float Cx = __fdiv_rn(2.f, __fmul_rn((float)W, i)), Cy = __fdiv_rn(2.f, __fmul_rn((float)H, j));
  const float D = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(Cy, Cy), d.dzx), d.dzx),
                                      __fmul_rn(__fmul_rn(__fmul_rn(Cx, Cx), d.dzy), d.dzy)),
                            __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(Cx, Cx), Cy), Cy), Z), Z));
  float3 n = make_float3(0.f, 0.f, 0.f);
  if (D != 0.f) {
    const float rv = __fdiv_rn(1.f, __fsqrt_rn(D));
    n = make_float3(__fmul_rn(__fmul_rn(-Cy, d.dzx), rv), __fmul_rn(__fmul_rn(-Cx, d.dzy), rv),
                    __fmul_rn(__fmul_rn(__fmul_rn(Cx, Cy), __fsub_rn(1.f, Z)), rv));
  }
  n = nrm(n);
  if (__fadd_rn(__fmul_rn(n.x, n.x), __fmul_rn(n.y, n.y)) > 1.f) {
    rgba[p] = bgc;
    return;
  }
  const float3 light = make_float3(0.f, -10.f, -1.f);
  const float3 li = make_float3(powf(0.252f, gamma), powf(0.212f, gamma), powf(0.15f, gamma));
  const float posx = __fmul_rn(__fsub_rn(i, 0.5f), 2.f), posy = __fmul_rn(__fsub_rn(j, 0.5f), 2.f);
  const float3 e0 = make_float3(__fmul_rn(Z, __fmul_rn(-posx, sh.p00)), __fmul_rn(Z, __fmul_rn(-posy, sh.p11)), Z);
  // vec4(eye, 1) * inverse(ModelView): row vector times matrix
  const float* m = sh.mv_inv.m;
  float3 eye;
  eye.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(e0.x, m[0]), __fmul_rn(e0.y, m[1])), __fmul_rn(e0.z, m[2])), m[3]);
  eye.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(e0.x, m[4]), __fmul_rn(e0.y, m[5])), __fmul_rn(e0.z, m[6])), m[7]);
  eye.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(e0.x, m[8]), __fmul_rn(e0.y, m[9])), __fmul_rn(e0.z, m[10])), m[11]);
  const float3 from_eye = nrm(eye);
  const float wc[3] = {powf(0.2f, gamma), powf(0.5f, gamma), powf(0.7f, gamma)};
  const float lambert = fmaxf(0.f, dot3f(nrm(light), n));
  const float cosine = fmaxf(0.f, dot3f(nrm(make_float3(__fsub_rn(light.x, eye.x), __fsub_rn(light.y, eye.y),
                                                        __fsub_rn(light.z, eye.z))), n));
  const float F = fminf(fmaxf(fresnel(1.0f, 1.33f, n, from_eye), 0.f), 1.f);
  const float ab = expf(-thickness);
  const float lt[3] = {li.x, li.y, li.z};
  float out[3];
  for (int c = 0; c < 3; ++c) {
    const float absorb = __fmul_rn(__fmul_rn(lt[c], __fadd_rn(wc[c], __fmul_rn(wc[c], cosine))), ab);
    const float surf = __fadd_rn(__fmul_rn(__fmul_rn(__fadd_rn(lambert, 0.2f), absorb), __fsub_rn(1.f, F)),
                                 __fdiv_rn(__fmul_rn(F, sh.env[c]), 2.f));
    const float mixed = __fadd_rn(__fmul_rn(surf, 0.5f), __fmul_rn(__fdiv_rn(sh.bg[c], 2.f), 0.5f));
    out[c] = powf(mixed, __fdiv_rn(1.f, gamma));
  }
  const float absorb_a = __fmul_rn(__fadd_rn(1.f, cosine), ab);
  const float surf_a = __fadd_rn(__fmul_rn(__fmul_rn(__fadd_rn(lambert, 0.2f), absorb_a), __fsub_rn(1.f, F)),
                                 __fdiv_rn(F, 2.f));
  rgba[p] = make_float4(out[0], out[1], out[2], __fadd_rn(__fmul_rn(surf_a, 0.5f), 0.25f));
}

bool invert4(const float* m, float* out) {  // general 4x4 inverse (cofactors), column-major
  double a[16], inv[16];
  for (int k = 0; k < 16; ++k) a[k] = m[k];
  inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
  inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
  inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
  inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
  inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
  inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
  inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
  inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
  inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
  inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
  inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
  inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
  inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
  inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
  inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
  inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
  const double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
  if (det == 0.0) return false;
  for (int k = 0; k < 16; ++k) out[k] = (float)(inv[k] / det);
  return true;
}

inline unsigned blocks_for(size_t n) { return (unsigned)((n + kRBlock - 1) / kRBlock); }

}  // namespace
}  // namespace sph

using namespace sph;

struct SphRenderer {
  int W = 0, H = 0;
  uint32_t nparticles = 0;  // capacity of the sprite array
  Proj* sprites = nullptr;
  int TX = 0, TY = 0;  // tiles of kTile x kTile pixels
  uint32_t T = 0;
  uint32_t *tcount = nullptr, *toff = nullptr, *tcursor = nullptr, *scan_tmp = nullptr;
  uint32_t* tlist = nullptr;     // per tile: particle indices of the sprites that reach it
  uint32_t* tscratch = nullptr;  // 2 words per list entry (long-list sorts)
  size_t tlist_cap = 0;
  uint32_t *tsort = nullptr, *tbig = nullptr, *counters = nullptr;
  unsigned long long* dcount = nullptr;  // (sprite, tile) pairs, covered fragments
  float *zbuf[2] = {nullptr, nullptr}, *thick = nullptr, *kern = nullptr;
  int kern_c = -1;
  uint32_t* total_host = nullptr;         // pinned: list entries
  unsigned long long* hcount = nullptr;   // pinned: dcount
  FoamSprite* foam = nullptr;      // two per particle
  uint32_t foam_cap = 0;           // particles the foam sprites hold
  uint32_t* foam_key = nullptr;    // per pixel: last foam fragment's sprite + 1
  cudaStream_t stream = nullptr;
  int sms = 1;
};

namespace {
void render_free(SphRenderer* r) {
  void* bufs[] = {r->sprites, r->tcount, r->toff, r->tcursor, r->scan_tmp, r->tlist, r->tscratch,
                  r->tsort, r->tbig, r->counters, r->dcount, r->zbuf[0], r->zbuf[1], r->thick, r->kern,
                  r->foam, r->foam_key};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (r->total_host) cudaFreeHost(r->total_host);
  if (r->hcount) cudaFreeHost(r->hcount);
}
template <class T>
int ralloc(T** p, size_t n, const char* what) {
  return cuda_check(cudaMalloc((void**)p, sizeof(T) * (n ? n : 1)), what);
}
}  // namespace

extern "C" {

int sph_render_create(int width, int height, SphRenderer** out) {
  if (!out || width <= 0 || height <= 0 || (size_t)width * height >= (1ull << 31))
    return fail(SPH_ERR_ARG, "render_create: bad size %dx%d", width, height);
  *out = nullptr;
  SphRenderer* r = new SphRenderer();
  r->W = width;
  r->H = height;
  const size_t P = (size_t)width * height;
  r->TX = (width + kTile - 1) / kTile;
  r->TY = (height + kTile - 1) / kTile;
  r->T = (uint32_t)r->TX * (uint32_t)r->TY;
  const size_t T = r->T;
  int rc = SPH_OK;
  if (rc == SPH_OK) rc = ralloc(&r->tcount, T + 1, "render: tile counts");
  if (rc == SPH_OK) rc = ralloc(&r->toff, T + 1, "render: tile offsets");
  if (rc == SPH_OK) rc = ralloc(&r->tcursor, T, "render: tile cursors");
  if (rc == SPH_OK) rc = ralloc(&r->scan_tmp, scan_scratch_words((uint32_t)(T + 1)), "render: scan scratch");
  if (rc == SPH_OK) rc = ralloc(&r->tsort, T, "render: sort list");  // every tile may need a sort
  if (rc == SPH_OK) rc = ralloc(&r->tbig, T, "render: long sort list");
  if (rc == SPH_OK) rc = ralloc(&r->counters, 2, "render: sort counters");
  if (rc == SPH_OK) rc = ralloc(&r->dcount, 2, "render: pair and fragment counts");
  if (rc == SPH_OK) rc = ralloc(&r->zbuf[0], P, "render: depth");
  if (rc == SPH_OK) rc = ralloc(&r->zbuf[1], P, "render: depth");
  if (rc == SPH_OK) rc = ralloc(&r->thick, P, "render: thickness");
  if (rc == SPH_OK) rc = cuda_check(cudaMallocHost((void**)&r->total_host, sizeof(uint32_t)), "render: host word");
  if (rc == SPH_OK)
    rc = cuda_check(cudaMallocHost((void**)&r->hcount, 2 * sizeof(unsigned long long)), "render: host counts");
  if (rc == SPH_OK) rc = cuda_check(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking), "render: stream");
  if (rc == SPH_OK)
    rc = cuda_check(cudaFuncSetAttribute(k_sort_big_cells, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(kBlockSortMax * sizeof(uint32_t))), "render: sort shared memory");
  if (rc == SPH_OK) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&r->sms, cudaDevAttrMultiProcessorCount, dev);
  }
  if (rc != SPH_OK) {
    render_free(r);
    if (r->stream) cudaStreamDestroy(r->stream);
    delete r;
    return rc;
  }
  *out = r;
  return SPH_OK;
}

int sph_render_destroy(SphRenderer* r) {
  if (!r) return SPH_OK;
  cudaStreamSynchronize(r->stream);
  render_free(r);
  cudaStreamDestroy(r->stream);
  delete r;
  return SPH_OK;
}

int sph_render_frame(SphRenderer* r, const SphRenderParams* rp, const sph_float4* pos, uint32_t n,
                     float* depth_out, float* thickness_out, sph_float4* rgba_out,
                     uint64_t* fragments) {
  if (!r || !rp || (!pos && n)) return fail(SPH_ERR_ARG, "render_frame: null argument");
  if (rp->method < 0 || rp->method > 2 || rp->iterations < 0 || rp->kernel_center < 0 ||
      rp->kernel_center > SPH_RENDER_MAX_KERNEL_CENTER)
    return fail(SPH_ERR_ARG, "render_frame: bad method/iterations/kernel_center");
  const int W = r->W, H = r->H;
  const size_t P = (size_t)W * H;
  cudaStream_t st = r->stream;
  Mat4 mv, pr;
  for (int k = 0; k < 16; ++k) {
    mv.m[k] = rp->modelview[k];
    pr.m[k] = rp->projection[k];
  }
  Shade sh;
  if (!invert4(rp->modelview, sh.mv_inv.m)) return fail(SPH_ERR_ARG, "render_frame: singular modelview");
  sh.p00 = rp->projection[0];
  sh.p11 = rp->projection[5];
  for (int c = 0; c < 3; ++c) {
    sh.env[c] = rp->env_color[c];
    sh.bg[c] = rp->background[c];
  }
  if (n > r->nparticles) {
    if (r->sprites) cudaFree(r->sprites);
    r->sprites = nullptr;
    r->nparticles = 0;
    SPH_TRY(ralloc(&r->sprites, n, "render: sprites"));
    r->nparticles = n;
  }
  // G-buffer: sprites and tile counts, scan, bin, sort each tile's list, resolve
  const uint32_t T = r->T;
  SPH_CUDA(cudaMemsetAsync(r->tcount, 0, sizeof(uint32_t) * (T + 1), st), "render: clear tile counts");
  SPH_CUDA(cudaMemsetAsync(r->dcount, 0, 2 * sizeof(unsigned long long), st), "render: clear counts");
  if (n)
    k_project<<<blocks_for(n), kRBlock, 0, st>>>((const float4*)pos, n, mv, pr, W, H, rp->point_radius,
                                                 rp->point_scale, r->sprites, r->tcount, r->TX, r->dcount);
  SPH_CUDA(cudaGetLastError(), "render: project");
  SPH_TRY(exclusive_scan(r->tcount, r->toff, T + 1, r->scan_tmp, st));
  SPH_CUDA(cudaMemcpyAsync(r->total_host, r->toff + T, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "render: total");
  SPH_CUDA(cudaMemcpyAsync(r->hcount, r->dcount, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st),
           "render: pairs");
  SPH_CUDA(cudaStreamSynchronize(st), "render: total");
  if (r->hcount[0] >= (1ull << 32))
    return fail(SPH_ERR_ARG, "render_frame: %llu sprite-tile pairs (at most 2^32 - 1)", r->hcount[0]);
  const size_t M = *r->total_host;
  if (M > r->tlist_cap) {
    if (r->tlist) cudaFree(r->tlist);
    if (r->tscratch) cudaFree(r->tscratch);
    r->tlist = r->tscratch = nullptr;
    r->tlist_cap = 0;
    SPH_TRY(ralloc(&r->tlist, M, "render: tile lists"));
    SPH_TRY(ralloc(&r->tscratch, 2 * M, "render: sort scratch"));
    r->tlist_cap = M;
  }
  if (M) {
    SPH_CUDA(cudaMemcpyAsync(r->tcursor, r->toff, sizeof(uint32_t) * T, cudaMemcpyDeviceToDevice, st), "render: cursors");
    k_bin<<<blocks_for(n), kRBlock, 0, st>>>(r->sprites, n, W, H, r->TX, r->tcursor, r->tlist);
    SPH_CUDA(cudaMemsetAsync(r->counters, 0, 2 * sizeof(uint32_t), st), "render: sort counters");
    k_find_cells<<<blocks_for(T), kRBlock, 0, st>>>(T, r->tcount, 1u, r->tsort, r->counters, r->tbig);
    k_sort_cells<<<8 * r->sms, kSortWarps * 32, 0, st>>>(r->toff, r->tcount, r->tlist, r->tsort, r->counters);
    k_sort_big_cells<<<r->sms, kBigThreads, kBlockSortMax * sizeof(uint32_t), st>>>(
        r->toff, r->tcount, r->tlist, r->tbig, r->counters + 1, r->tscratch);
  }
  k_tile_resolve<<<T, kTilePixels, 0, st>>>(r->sprites, r->tlist, r->toff, r->tcount, W, H, r->TX, r->zbuf[0],
                                            r->thick, r->dcount + 1);
  SPH_CUDA(cudaGetLastError(), "render: g-buffer");
  // smoothing
  int cur = 0;
  if (rp->method == 2 && rp->kernel_center != r->kern_c) {
    float k[2 * SPH_RENDER_MAX_KERNEL_CENTER + 1];
    for (int i = -rp->kernel_center; i <= rp->kernel_center; ++i)
      k[rp->kernel_center + i] = (float)exp(-i * i * 0.1);  // CreateFilter (render_particles.cpp:724-728)
    if (!r->kern) SPH_TRY(ralloc(&r->kern, 2 * SPH_RENDER_MAX_KERNEL_CENTER + 1, "render: kernel"));
    SPH_CUDA(cudaMemcpyAsync(r->kern, k, sizeof(float) * (2 * rp->kernel_center + 1), cudaMemcpyHostToDevice, st), "render: kernel");
    SPH_CUDA(cudaStreamSynchronize(st), "render: kernel");
    r->kern_c = rp->kernel_center;
  }
  for (int it = 0; rp->method != 0 && it < rp->iterations; ++it) {
    if (rp->method == 1)
      k_curvature<<<blocks_for(P), kRBlock, 0, st>>>(r->zbuf[cur], r->zbuf[1 - cur], W, H);
    else
      k_bilateral<<<blocks_for(P), kRBlock, 0, st>>>(r->zbuf[cur], r->zbuf[1 - cur], W, H, r->kern,
                                                     rp->kernel_center, rp->sigma);
    cur = 1 - cur;
  }
  SPH_CUDA(cudaGetLastError(), "render: smoothing");
  if (rgba_out)
    k_shade<<<blocks_for(P), kRBlock, 0, st>>>(r->zbuf[cur], r->thick, W, H, sh, (float4*)rgba_out);
  if (depth_out)
    SPH_CUDA(cudaMemcpyAsync(depth_out, r->zbuf[cur], sizeof(float) * P, cudaMemcpyDeviceToDevice, st), "render: depth out");
  if (thickness_out)
    SPH_CUDA(cudaMemcpyAsync(thickness_out, r->thick, sizeof(float) * P, cudaMemcpyDeviceToDevice, st), "render: thickness out");
  SPH_CUDA(cudaGetLastError(), "render: shade");
  SPH_CUDA(cudaMemcpyAsync(r->hcount + 1, r->dcount + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st),
           "render: fragments");
  SPH_TRY(cuda_check(cudaStreamSynchronize(st), "render: frame"));
  if (fragments) *fragments = r->hcount[1];
  return SPH_OK;
}

int sph_render_foam(SphRenderer* r, const SphRenderParams* rp, const sph_float4* pos, const sph_float4* color,
                    uint32_t n, sph_float4* rgba_inout, float* foam_depth_out) {
  if (!r || !rp || ((!pos || !color) && n)) return fail(SPH_ERR_ARG, "render_foam: null argument");
  if (n > (1u << 30)) return fail(SPH_ERR_ARG, "render_foam: %u particles (at most 2^30)", n);
  const int W = r->W, H = r->H;
  const size_t P = (size_t)W * H;
  cudaStream_t st = r->stream;
  Mat4 mv, pr;
  for (int k = 0; k < 16; ++k) {
    mv.m[k] = rp->modelview[k];
    pr.m[k] = rp->projection[k];
  }
  if (!r->foam_key) SPH_TRY(ralloc(&r->foam_key, P, "render: foam keys"));
  if (n > r->foam_cap) {
    if (r->foam) cudaFree(r->foam);
    r->foam = nullptr;
    r->foam_cap = 0;
    SPH_TRY(ralloc(&r->foam, 2 * (size_t)n, "render: foam sprites"));
    r->foam_cap = n;
  }
  SPH_CUDA(cudaMemsetAsync(r->foam_key, 0, sizeof(uint32_t) * P, st), "render: clear foam keys");
  if (n) {
    k_foam_project<<<blocks_for(n), kRBlock, 0, st>>>((const float4*)pos, (const float4*)color, n, mv, pr, W, H,
                                                      rp->point_radius, rp->point_scale, r->foam);
    k_foam_cover<<<blocks_for(2 * (size_t)n), kRBlock, 0, st>>>(r->foam, 2 * n, W, H, r->foam_key);
  }
  if (rgba_inout || foam_depth_out)
    k_foam_resolve<<<blocks_for(P), kRBlock, 0, st>>>(r->foam, r->foam_key, W, H, pr, (float4*)rgba_inout,
                                                      foam_depth_out);
  SPH_CUDA(cudaGetLastError(), "render: foam");
  return cuda_check(cudaStreamSynchronize(st), "render: foam");
}

}  // extern "C"
