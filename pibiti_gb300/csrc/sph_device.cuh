// sph_device.cuh -- per-particle device math shared by every SPH kernel.
//
// Each function restates one piece of the reference's device code (cited on
// the function).  The translation units that include this header are built
// with --fmad=false, so every multiply and add rounds separately exactly as
// written; the few fused multiply-adds are explicit __fmaf_rn calls, and
// divisions and square roots are the IEEE round-to-nearest intrinsics.  The
// arithmetic is therefore a fixed sequence of IEEE operations.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "sph_params.h"

namespace sph {

constexpr uint32_t kEmpty = 0xffffffffu;

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float len3(float3 a) { return __fsqrt_rn(dot3(a, a)); }
__device__ __forceinline__ float len2(float x, float y) {
  return __fsqrt_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)));
}

// __mul24 semantics: product of the low 24 bits of each operand, signed.
__device__ __forceinline__ int mul24(int a, int b) { return __mul24(a, b); }

// calcGridPos (Kernel_Cell.cui:5-13): floor((p - worldMin) / cellSize).
// float->int conversion saturates and maps NaN to 0, as cvt.rmi does.
__device__ __forceinline__ int3 grid_pos(const SimParams& p, float4 x) {
  const float gx = __fdiv_rn(__fsub_rn(x.x, p.worldMin.x), p.cellSize.x);
  const float gy = __fdiv_rn(__fsub_rn(x.y, p.worldMin.y), p.cellSize.y);
  const float gz = __fdiv_rn(__fsub_rn(x.z, p.worldMin.z), p.cellSize.z);
  return make_int3(__float2int_rd(gx), __float2int_rd(gy), __float2int_rd(gz));
}

// calcGridHash (Kernel_Cell.cui:15-19), including its wrap-around for
// coordinates outside the grid.
__device__ __forceinline__ uint32_t grid_hash_raw(const SimParams& p, int x, int y, int z) {
  return (uint32_t)(mul24(z, (int)p.gridSize_yx) + mul24(y, (int)p.gridSize.x) + x);
}

// Cell index of a position, clamped into the grid.  Identical to the raw hash
// for every position inside the world box; a position outside it (only
// possible for NaN or for data placed outside the box by the caller) lands in
// the nearest cell instead of an aliased or out-of-range one.
__device__ __forceinline__ uint32_t cell_of(const SimParams& p, int3 g) {
  const int x = min(max(g.x, 0), (int)p.gridSize.x - 1);
  const int y = min(max(g.y, 0), (int)p.gridSize.y - 1);
  const int z = min(max(g.z, 0), (int)p.gridSize.z - 1);
  return (uint32_t)(z * (int)p.gridSize_yx + y * (int)p.gridSize.x + x);
}

// One soft wall of boundary() (System.cu:52-53, addB/addC):
// acc = stiff*diff - damp*dot(n, v); v += acc * n * dt.
__device__ __forceinline__ void add_wall(float3& v, float3 n, float diff, float stiff, float damp,
                                         float dt) {
  const float acc = __fsub_rn(__fmul_rn(stiff, diff), __fmul_rn(damp, dot3(n, v)));
  v.x = __fadd_rn(v.x, __fmul_rn(__fmul_rn(acc, n.x), dt));
  v.y = __fadd_rn(v.y, __fmul_rn(__fmul_rn(acc, n.y), dt));
  v.z = __fadd_rn(v.z, __fmul_rn(__fmul_rn(acc, n.z), dt));
}

// boundary() (System.cu:41-159): every boundary type and z effect.
__device__ inline void boundary(const SimParams& p, float3& pos, float3& vel) {
  float3 wmin = p.worldMin, wmax = p.worldMax;
  const float b = p.distBndSoft, stiff = p.bndStiff, damp = p.bndDamp, damp2 = p.bndDampC;
  const float dt = p.timeStep;
  const float EPS = 0.00001f;
  const uint32_t t = p.bndType;
  const bool bCylY = t == SPH_BND_CYL_Y, bCylZ = t == SPH_BND_CYL_Z;
  const bool bWave = p.bndEffZ == SPH_BND_EFF_WAVE, bNoEff = p.bndEffZ == SPH_BND_EFF_NONE,
             bCycle = p.bndEffZ == SPH_BND_EFF_CYCLE;
  float diff;
  if (bWave) {
    const float sl = -p.r2Angle;
    diff = __fsub_rn(__fsub_rn(b, __fsub_rn(pos.y, wmin.y)), __fmul_rn(__fsub_rn(pos.z, wmin.z), sl));
    if (diff > EPS) add_wall(vel, f3(0.f, __fsub_rn(1.f, sl), sl), diff, stiff, damp, dt);
    wmin.z = __fadd_rn(wmin.z, __fmul_rn(p.rTwist, __fadd_rn(1.f, sinf(p.rAngle))));
  }
  if (t != SPH_BND_SPHERE) {
    if (!bCylY) {
      if (bNoEff || bWave) {
        diff = __fadd_rn(__fsub_rn(b, pos.z), wmin.z);
        if (diff > EPS) add_wall(vel, f3(0.f, 0.f, 1.f), diff, stiff, damp2, dt);
      }
      if (!bCycle) {
        diff = __fsub_rn(__fadd_rn(b, pos.z), wmax.z);
        if (diff > EPS) add_wall(vel, f3(0.f, 0.f, -1.f), diff, stiff, damp2, dt);
      }
    }
    if (!bCylY && !bCylZ) {
      diff = __fadd_rn(__fsub_rn(b, pos.x), wmin.x);
      if (diff > EPS) add_wall(vel, f3(1.f, 0.f, 0.f), diff, stiff, damp, dt);
      diff = __fsub_rn(__fadd_rn(b, pos.x), wmax.x);
      if (diff > EPS) add_wall(vel, f3(-1.f, 0.f, 0.f), diff, stiff, damp, dt);
    }
    if (!bCylZ) {
      diff = __fadd_rn(__fsub_rn(b, pos.y), wmin.y);
      if (diff > EPS) add_wall(vel, f3(0.f, 1.f, 0.f), diff, stiff, damp, dt);
      diff = __fsub_rn(__fadd_rn(b, pos.y), wmax.y);
      if (diff > EPS) add_wall(vel, f3(0.f, -1.f, 0.f), diff, stiff, damp, dt);
    }
  } else {
    const float len = len3(pos);
    diff = __fadd_rn(__fadd_rn(b, len), wmin.y);
    if (diff > EPS)
      add_wall(vel, f3(__fdiv_rn(-pos.x, len), __fdiv_rn(-pos.y, len), __fdiv_rn(-pos.z, len)),
               diff, stiff, damp2, dt);
  }
  if (bCylY || t == SPH_BND_CYL_YZ) {
    const float len = len2(pos.x, pos.z);
    diff = __fsub_rn(__fadd_rn(b, len), wmax.x);
    if (diff > EPS)
      add_wall(vel, f3(__fdiv_rn(-pos.x, len), 0.f, __fdiv_rn(-pos.z, len)), diff, stiff, damp2, dt);
  }
  if (bCylZ || t == SPH_BND_CYL_YZ) {
    const float len = len2(pos.x, pos.y);
    diff = __fadd_rn(__fadd_rn(b, len), wmin.y);
    if (diff > EPS)
      add_wall(vel, f3(__fdiv_rn(-pos.x, len), __fdiv_rn(-pos.y, len), 0.f), diff, stiff, damp2, dt);
  }
  if (!bWave && !bNoEff) {
    const float dr = __fmul_rn(1.f, p.particleR);
    const float span = __fsub_rn(__fsub_rn(__fsub_rn(wmax.z, wmin.z), __fmul_rn(2.f, b)), dr);
    if (bCycle && vel.z > p.rVexit && pos.z > __fsub_rn(__fsub_rn(wmax.z, b), dr))
      pos.z = __fsub_rn(pos.z, span);
    else if (vel.z < -p.rVexit && pos.z < __fadd_rn(__fadd_rn(wmin.z, b), dr))
      pos.z = __fadd_rn(pos.z, span);
  }
  if (t == SPH_BND_PUMP_Y) {
    const float PI2_ = 2.f * 3.141592654f;
    const float rad = wmax.x, ang = p.angOut, hc = p.hClose, rin = __fmul_rn(rad, p.radIn);
    const float len = len2(pos.x, pos.y);
    const float3 nrad = f3(__fdiv_rn(-pos.x, len), __fdiv_rn(-pos.y, len), 0.f);
    diff = __fsub_rn(__fadd_rn(b, len), rad);
    if (diff > EPS) {
      const float a = atanf(__fdiv_rn(pos.x, pos.y));
      if (ang < 0.5f) {
        if (a < -ang || a > ang || pos.y < 0) add_wall(vel, nrad, diff, stiff, damp, dt);
      } else {
        if (pos.y < 0 || (len < __fmul_rn(rad, p.s5) && a < ang)) add_wall(vel, nrad, diff, stiff, damp, dt);
      }
    }
    float xs;
    if (ang < 0.5f) {
      xs = __fmul_rn(sinf(__fmul_rn(ang, p.s3)), rad);
      const float zs = __fmul_rn(__fmul_rn(cosf(__fmul_rn(ang, p.s3)), rad), p.s4);
      if (pos.y > zs) {
        diff = __fsub_rn(__fsub_rn(b, pos.x), xs);
        if (diff > EPS) add_wall(vel, f3(1.f, 0.f, 0.f), diff, stiff, damp, dt);
        diff = __fsub_rn(__fadd_rn(b, pos.x), xs);
        if (diff > EPS) add_wall(vel, f3(-1.f, 0.f, 0.f), diff, stiff, damp, dt);
      }
    } else {
      xs = __fmul_rn(0.09f, p.s4);
      if (len >= __fmul_rn(rad, p.s6)) {
        diff = __fadd_rn(__fsub_rn(b, pos.x), xs);
        if (diff > EPS) add_wall(vel, f3(1.f, 0.f, 0.f), diff, stiff, damp, dt);
      }
    }
    if (pos.z > __fsub_rn(hc, __fmul_rn(b, p.s1))) {
      diff = __fsub_rn(__fadd_rn(b, len), rin);
      if (diff > EPS) add_wall(vel, nrad, diff, stiff, damp, dt);
    }
    if (pos.z < __fsub_rn(hc, __fmul_rn(b, p.s2))) {
      diff = __fsub_rn(__fadd_rn(b, pos.z), hc);
      if (diff > EPS) add_wall(vel, f3(0.f, 0.f, -1.f), diff, stiff, damp, dt);
    }
    diff = __fadd_rn(__fsub_rn(pos.y, wmax.y), p.rDexit);
    if (diff > EPS && vel.y > p.rVexit) {
      float aa, rr;
      const float zz = fabsf(__fsub_rn(hc, wmin.z));
      if (ang < 0.5f) {
        const float xx = __fmul_rn(xs, 2.f);
        rr = __fmul_rn(__fdiv_rn(__fadd_rn(pos.x, __fdiv_rn(xx, 2.f)), xx), 0.7f);
        aa = __fmul_rn(__fdiv_rn(__fsub_rn(pos.z, __fdiv_rn(zz, 2.f)), zz), 1.6f);
      } else {
        rr = __fmul_rn(__fdiv_rn(__fsub_rn(wmax.x, pos.x), xs), 0.45f);
        aa = __fmul_rn(__fdiv_rn(__fsub_rn(pos.z, __fdiv_rn(zz, 2.f)), zz), 1.8f);
      }
      rr = __fmul_rn(rr, rin);
      aa = __fmul_rn(aa, PI2_);
      const float x = __fmul_rn(cosf(aa), rr), y = __fmul_rn(sinf(aa), rr);
      const float z = (float)__dsub_rn((double)__fsub_rn(wmax.z, b),
                                       __dmul_rn((double)fabsf(__fsub_rn(vel.y, p.rVexit)), 0.01));
      pos = f3(x, y, z);
      vel = f3(vel.x, vel.z, -vel.y);
    }
  }
}

// integrateD (System.cu:165-205): boundary, v += g dt, v *= damping,
// x += v dt, hard clamp.  w components are carried by the caller.
__device__ __forceinline__ void integrate(const SimParams& p, float3& x, float3& v) {
  boundary(p, x, v);
  const float dt = p.timeStep, damp = p.globalDamping;
  v.x = __fadd_rn(v.x, __fmul_rn(p.gravity.x, dt));
  v.y = __fadd_rn(v.y, __fmul_rn(p.gravity.y, dt));
  v.z = __fadd_rn(v.z, __fmul_rn(p.gravity.z, dt));
  v.x = __fmul_rn(v.x, damp);
  v.y = __fmul_rn(v.y, damp);
  v.z = __fmul_rn(v.z, damp);
  x.x = __fadd_rn(x.x, __fmul_rn(v.x, dt));
  x.y = __fadd_rn(x.y, __fmul_rn(v.y, dt));
  x.z = __fadd_rn(x.z, __fmul_rn(v.z, dt));
  const float b = p.distBndHard;
  const float hix = __fsub_rn(p.worldMax.x, b), lox = __fadd_rn(p.worldMin.x, b);
  const float hiy = __fsub_rn(p.worldMax.y, b), loy = __fadd_rn(p.worldMin.y, b);
  const float hiz = __fsub_rn(p.worldMax.z, b), loz = __fadd_rn(p.worldMin.z, b);
  if (x.x > hix) x.x = hix;
  if (x.x < lox) x.x = lox;
  if (x.y > hiy) x.y = hiy;
  if (x.y < loy) x.y = loy;
  if (x.z > hiz) x.z = hiz;
  if (x.z < loz) x.z = loz;
}

// Pair term of compDensCell (Kernel_Cell.cui:157-169): (h^2 - r^2)^3 when
// r^2 < h^2, accumulated as acc + (c*c)*c with one fused step.
__device__ __forceinline__ float density_pair(float4 a, float4 b, float h2, float acc, int& nbr) {
  const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
  const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
  if (r2 < h2) {
    const float c = __fsub_rn(h2, r2);
    acc = __fmaf_rn(__fmul_rn(c, c), c, acc);
    ++nbr;
  }
  return acc;
}

// Constants of compForcePair hoisted out of the neighbour loop.  h2_out is
// two ulps above fl(h*h): a squared distance at or above it has a correctly
// rounded square root >= h, so the pair contributes nothing (r < h fails)
// and can be skipped before the division and square root.
struct ForceConsts {
  float h, minDist, spiky, vterm, minDens, h2_out;
};
__device__ __forceinline__ ForceConsts force_consts(const SimParams& p) {
  ForceConsts k;
  k.h = p.h;
  k.minDist = p.minDist;
  k.spiky = p.SpikyKern;
  k.vterm = __fmul_rn(p.LapKern, p.viscosity);
  k.minDens = p.minDens;
  k.h2_out = __int_as_float(__float_as_int(__fmul_rn(p.h, p.h)) + 2);
  return k;
}

__device__ __forceinline__ void force_pair_near(const ForceConsts& k, float4 vi, float inv_di,
                                                float pi, float4 vj, float inv_dj, float pj,
                                                float rx, float ry, float rz, float dist2,
                                                float3& acc);

// compForceCell inner step + compForcePair (Kernel_Cell.cui:210-228,
// 251-258): d12 = min(minDens, 1/(rho_i rho_j)); r = max(minDist, |x_i-x_j|);
// if r < h: F += (c Spiky (p_i+p_j)/r (x_i-x_j) + Lap mu (v_j-v_i)) c d12.
// 1/(rho_i rho_j) is formed as (1/rho_i)(1/rho_j) from the correctly
// rounded reciprocals, so that a walk computes one per particle and none
// per pair (within 2 ulp of the reference's single division).
__device__ __forceinline__ void force_pair(const ForceConsts& k, float4 xi, float4 vi, float inv_di,
                                           float pi, float4 xj, float4 vj, float inv_dj, float pj,
                                           float3& acc) {
  const float rx = __fsub_rn(xi.x, xj.x), ry = __fsub_rn(xi.y, xj.y), rz = __fsub_rn(xi.z, xj.z);
  const float dist2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx)));
  force_pair_near(k, vi, inv_di, pi, vj, inv_dj, pj, rx, ry, rz, dist2, acc);
}

// The pair term after the squared distance: returns whether r < h and then
// sets f; the caller adds f to the cell's partial sum.
__device__ __forceinline__ bool force_term(const ForceConsts& k, float4 vi, float inv_di, float pi,
                                           float4 vj, float inv_dj, float pj, float rx, float ry,
                                           float rz, float dist2, float3& f) {
  const float dd = __fmul_rn(inv_di, inv_dj);
  const float d12 = fminf(k.minDens, dd);
  const float vx = __fsub_rn(vj.x, vi.x), vy = __fsub_rn(vj.y, vi.y), vz = __fsub_rn(vj.z, vi.z);
  const float r = fmaxf(k.minDist, __fsqrt_rn(dist2));
  const float c = __fsub_rn(k.h, r);
  const float pterm = __fdiv_rn(__fmul_rn(__fmul_rn(c, k.spiky), __fadd_rn(pi, pj)), r);
  const float s = __fmul_rn(c, d12);
  f.x = __fmul_rn(__fmaf_rn(pterm, rx, __fmul_rn(k.vterm, vx)), s);
  f.y = __fmul_rn(__fmaf_rn(pterm, ry, __fmul_rn(k.vterm, vy)), s);
  f.z = __fmul_rn(__fmaf_rn(pterm, rz, __fmul_rn(k.vterm, vz)), s);
  return r < k.h;
}

// force_term with the x and y components as FP32 pairs (sm_100+ packed
// instructions; each half rounds as the scalar _rn operation): vj - vi as
// fma(vi, -1, vj), which is the IEEE difference with the same signed zeros,
// and the force's x and y in one multiply, fma and multiply each.  Same
// result bits as force_term.
__device__ __forceinline__ bool force_term_xy(const ForceConsts& k, float2 vi_xy, float vi_z, float inv_di,
                                              float pi, float4 vj, float inv_dj, float pj, float2 r_xy,
                                              float rz, float dist2, float2& f_xy, float& f_z) {
  const float dd = __fmul_rn(inv_di, inv_dj);
  const float d12 = fminf(k.minDens, dd);
  const float2 v_xy = __ffma2_rn(vi_xy, make_float2(-1.f, -1.f), make_float2(vj.x, vj.y));
  const float vz = __fsub_rn(vj.z, vi_z);
  const float r = fmaxf(k.minDist, __fsqrt_rn(dist2));
  const float c = __fsub_rn(k.h, r);
  const float pterm = __fdiv_rn(__fmul_rn(__fmul_rn(c, k.spiky), __fadd_rn(pi, pj)), r);
  const float s = __fmul_rn(c, d12);
  const float2 t = __ffma2_rn(make_float2(pterm, pterm), r_xy,
                              __fmul2_rn(make_float2(k.vterm, k.vterm), v_xy));
  f_xy = __fmul2_rn(t, make_float2(s, s));
  f_z = __fmul_rn(__fmaf_rn(pterm, rz, __fmul_rn(k.vterm, vz)), s);
  return r < k.h;
}

// The part of force_pair after the squared distance; the fused walk calls it
// only for candidates not excluded by ForceConsts::h2_out (and for NaN).
__device__ __forceinline__ void force_pair_near(const ForceConsts& k, float4 vi, float inv_di,
                                                float pi, float4 vj, float inv_dj, float pj,
                                                float rx, float ry, float rz, float dist2,
                                                float3& acc) {
  float3 f;
  if (force_term(k, vi, inv_di, pi, vj, inv_dj, pj, rx, ry, rz, dist2, f)) {
    acc.x = __fadd_rn(acc.x, f.x);
    acc.y = __fadd_rn(acc.y, f.y);
    acc.z = __fadd_rn(acc.z, f.z);
  }
}

// collideSpheres (Kernel_Cell.cui:78-96); float3/float is a multiply by the
// reciprocal (cutil_math.h:358-362).
__device__ __forceinline__ float3 collide_sphere(const SimParams& p, float3 rel, float3 rv,
                                                 float radius) {
  const float dist = len3(rel);
  float3 f = f3(0.f, 0.f, 0.f);
  if (dist < radius) {
    const float inv = __fdiv_rn(1.0f, dist);
    const float3 n = f3(__fmul_rn(rel.x, inv), __fmul_rn(rel.y, inv), __fmul_rn(rel.z, inv));
    const float vn = dot3(rv, n);
    const float3 tv = f3(__fsub_rn(rv.x, __fmul_rn(vn, n.x)), __fsub_rn(rv.y, __fmul_rn(vn, n.y)),
                         __fsub_rn(rv.z, __fmul_rn(vn, n.z)));
    const float sp = __fmul_rn(p.spring, __fsub_rn(dist, radius));
    f.x = __fadd_rn(__fadd_rn(__fmul_rn(sp, n.x), __fmul_rn(p.damping, rv.x)), __fmul_rn(p.shear, tv.x));
    f.y = __fadd_rn(__fadd_rn(__fmul_rn(sp, n.y), __fmul_rn(p.damping, rv.y)), __fmul_rn(p.shear, tv.y));
    f.z = __fadd_rn(__fadd_rn(__fmul_rn(sp, n.z), __fmul_rn(p.damping, rv.z)), __fmul_rn(p.shear, tv.z));
  }
  return f;
}

// collideSpheresR (Kernel_Cell.cui:101-115): spring and damping only.
__device__ __forceinline__ float3 collide_sphere_r(const SimParams& p, float3 rel, float3 rv,
                                                   float radius) {
  const float dist = len3(rel);
  float3 f = f3(0.f, 0.f, 0.f);
  if (dist < radius) {
    const float inv = __fdiv_rn(1.0f, dist);
    const float3 n = f3(__fmul_rn(rel.x, inv), __fmul_rn(rel.y, inv), __fmul_rn(rel.z, inv));
    const float sp = __fmul_rn(p.spring, __fsub_rn(dist, radius));
    f.x = __fadd_rn(__fmul_rn(sp, n.x), __fmul_rn(p.damping, rv.x));
    f.y = __fadd_rn(__fmul_rn(sp, n.y), __fmul_rn(p.damping, rv.y));
    f.z = __fadd_rn(__fmul_rn(sp, n.z), __fmul_rn(p.damping, rv.z));
  }
  return f;
}

__device__ __forceinline__ void add3(float3& a, float3 b) {
  a.x = __fadd_rn(a.x, b.x);
  a.y = __fadd_rn(a.y, b.y);
  a.z = __fadd_rn(a.z, b.z);
}

// Height-map collider (System.cu:253-309): collision spheres on a sine
// surface over the XZ plane (iHmap == 1) or the YZ plane, 5 x 5 x 2 around
// the particle.
__device__ inline void heightmap(const SimParams& p, float4 xi, float4 vi, float3& add) {
  const float PI_ = 3.141592654f;
  const float3 vel3 = f3(-vi.x, -vi.y, -vi.z);
  const float rr = __fadd_rn(p.particleR, p.rotR), spc = p.rotSpc;
  const float o2 = __fdiv_rn(__fmul_rn(p.s2, PI_), 180.f), o4 = __fdiv_rn(__fmul_rn(p.s4, PI_), 180.f);
  const bool xz = p.iHmap == 1;
  // (u, z) plane coordinates: u is x for the XZ map, y for the YZ map
  const float pu = xz ? xi.x : xi.y, umin = xz ? p.worldMin.x : p.worldMin.y;
  const float usz = xz ? p.worldSizeD.x : p.worldSizeD.y;
  const float hmin = xz ? p.worldMin.y : p.worldMin.x;
  const int iu = __float2int_rz(__fdiv_rn(__fsub_rn(pu, umin), spc));
  const float uf = __fadd_rn(__fmul_rn((float)iu, spc), umin);
  const int iz = __float2int_rz(__fdiv_rn(__fsub_rn(xi.z, p.worldMin.z), spc));
  const float zf = __fadd_rn(__fmul_rn((float)iz, spc), p.worldMin.z);
#pragma unroll 1
  for (int j = -2; j <= 2; ++j)
#pragma unroll 1
    for (int i = -2; i <= 2; ++i) {
      const float uh = __fadd_rn(uf, __fmul_rn((float)i, spc));
      const float zh = __fadd_rn(zf, __fmul_rn((float)j, spc));
      for (int k = 0; k <= 1; ++k) {
        const float un = __fmul_rn(__fmul_rn(__fdiv_rn(uh, usz), 2.f), PI_);
        const float zn = __fmul_rn(__fmul_rn(__fdiv_rn(zh, p.worldSizeD.z), 2.f), PI_);
        const float ss = __fmul_rn(sinf(__fadd_rn(__fmul_rn(p.s1, un), o2)),
                                   sinf(__fadd_rn(__fmul_rn(p.s3, zn), o4)));
        if (p.s5 <= -1.f || ss > p.s5) {
          const float hf = __fadd_rn(__fadd_rn(__fmul_rn(ss, p.hClose), p.r2Angle), hmin);
          const float hh = __fsub_rn(hf, __fmul_rn((float)k, spc));
          const float3 rel = xz ? f3(__fsub_rn(uh, xi.x), __fsub_rn(hh, xi.y), __fsub_rn(zh, xi.z))
                                : f3(__fsub_rn(hh, xi.x), __fsub_rn(uh, xi.y), __fsub_rn(zh, xi.z));
          add3(add, collide_sphere_r(p, rel, vel3, rr));
        }
      }
    }
}

// Rotor and propeller colliders (System.cu:311-372): rotType 1 (pump rotor
// about z), 2 (pump rotor about y), 3 (propeller about z, optionally two).
__device__ inline void rotor(const SimParams& p, float4 xi, float4 vi, float3& add) {
  const float PI_ = 3.141592654f;
  const int sx = p.rotSize.x, sy = p.rotSize.y, sz = p.rotSize.z, cb = p.rotBlades;
  const float sp = p.rotSpc, ca = __fdiv_rn(__fmul_rn(2.f, PI_), (float)cb);
  const float x2 = __fmul_rn((float)sx, 0.5f), y2 = __fmul_rn((float)sy, 0.5f);
  const float rr = __fadd_rn(p.particleR, p.rotR);
  const float3 vel3 = f3(-vi.x, -vi.y, -vi.z);
  const float cx = p.collPos.x, cy = p.collPos.y, cz = p.collPos.z;
  if (p.rotType == 1 || p.rotType == 2) {
    const bool zrot = p.rotType == 1;
    const float pa = zrot ? xi.z : xi.y, ca0 = zrot ? cz : cy;
    if (!(pa > __fsub_rn(ca0, rr) && pa < __fadd_rn(__fadd_rn(ca0, rr), __fmul_rn(sp, (float)sy))))
      return;
#pragma unroll 1
    for (int z = 1; z <= sz; ++z)
#pragma unroll 1
      for (int x = 0; x <= sx; ++x)
#pragma unroll 1
        for (int c = 0; c < cb; ++c) {
          const float a = __fadd_rn(__fadd_rn(-p.rAngle, __fmul_rn((float)c, ca)),
                                    __fmul_rn((float)z, p.rTwist));
          const float cs = __fmul_rn(cosf(a), sp), sn = __fmul_rn(-sinf(a), sp);
          const float xx = __fsub_rn((float)x, x2);
          const float q0 = __fsub_rn(__fmul_rn(xx, cs), __fmul_rn((float)z, sn));
          const float q1 = __fadd_rn(__fmul_rn(xx, sn), __fmul_rn((float)z, cs));
#pragma unroll 1
          for (int y = 0; y <= sy; ++y) {
            const float qy = __fmul_rn(sp, (float)y);
            const float3 rel =
                zrot ? f3(__fsub_rn(__fadd_rn(cx, q0), xi.x), __fsub_rn(__fadd_rn(cy, q1), xi.y),
                          __fsub_rn(__fadd_rn(cz, qy), xi.z))
                     : f3(__fsub_rn(__fadd_rn(cx, q0), xi.x), __fsub_rn(__fadd_rn(cy, qy), xi.y),
                          __fsub_rn(__fadd_rn(cz, q1), xi.z));
            add3(add, collide_sphere_r(p, rel, vel3, rr));
          }
        }
  } else if (p.rotType == 3) {
    const float half = __fdiv_rn(__fmul_rn(sp, (float)sz), 2.f);
    if (!(xi.z > __fsub_rn(__fsub_rn(cz, rr), half) && xi.z < __fadd_rn(__fadd_rn(cz, rr), half))) return;
    float rx = cx, aa = p.rAngle, tw = p.rTwist;
    if (p.r2Dist > 0.f) {
      if (xi.x > 0.f) {
        rx = __fadd_rn(rx, __fmul_rn(p.r2Dist, 0.5f));
      } else {
        rx = __fsub_rn(rx, __fmul_rn(p.r2Dist, 0.5f));
        aa = p.r2Angle;
        tw = __fmul_rn(tw, p.r2twist);
      }
    }
#pragma unroll 1
    for (int c = 0; c < cb; ++c) {
      const float a = __fadd_rn(aa, __fmul_rn((float)c, ca));
#pragma unroll 1
      for (int h = 0; h <= sy; ++h) {
        float dh = 0.f;
        if (h == sy - 1) dh = 0.5f;
        else if (h == sy) dh = 1.2f;
#pragma unroll 1
        for (int x = 0; x <= sz; ++x) {
          float d = dh;
          if (x == sz && d == 0.f) d = 0.4f;
          const float k = cosf(__fadd_rn(__fmul_rn(__fsub_rn((float)x, x2), 0.2f), __fmul_rn(PI_, 0.6f)));
          const float at = __fmul_rn(tw, __fsub_rn(__fmul_rn(d, -0.05f), __fmul_rn(__fsub_rn((float)h, y2), k)));
          const float ac = __fadd_rn(a, at);
          const float cs = __fmul_rn(cosf(ac), sp), sn = __fmul_rn(-sinf(ac), sp);
          const float qx = __fmul_rn((float)x, cs), qy = __fmul_rn((float)x, sn);
          const float qz = __fmul_rn(__fmul_rn(sp, __fsub_rn(__fadd_rn(-d, (float)h), y2)), k);
          const float r = __fmul_rn(p.rotR, fabsf(__fsub_rn(1.f, d)));
          const float3 rel = f3(__fsub_rn(__fadd_rn(rx, qx), xi.x), __fsub_rn(__fadd_rn(cy, qy), xi.y),
                                __fsub_rn(__fadd_rn(cz, qz), xi.z));
          add3(add, collide_sphere_r(p, rel, vel3, __fadd_rn(p.particleR, r)));
        }
      }
    }
  }
}

// The part of computeForceD after the neighbour sums (System.cu:249-250,
// 253-402): dv = F m dt, the height map, the rotor or the sphere collider,
// and the accelerators.
__device__ inline float3 velocity_increment(const SimParams& p, float3 F, float4 xi, float4 vi) {
  const float s = __fmul_rn(p.particleMass, p.timeStep);
  float3 add = f3(__fmul_rn(F.x, s), __fmul_rn(F.y, s), __fmul_rn(F.z, s));
  if (p.iHmap > 0) heightmap(p, xi, vi, add);
  if (p.rotType > 0) {
    rotor(p, xi, vi, add);
  } else {
    const float3 rel = f3(__fsub_rn(p.collPos.x, xi.x), __fsub_rn(p.collPos.y, xi.y),
                          __fsub_rn(p.collPos.z, xi.z));
    const float3 c = collide_sphere(p, rel, f3(-vi.x, -vi.y, -vi.z), __fadd_rn(p.particleR, p.collR));
    add.x = __fadd_rn(add.x, c.x);
    add.y = __fadd_rn(add.y, c.y);
    add.z = __fadd_rn(add.z, c.z);
  }
#pragma unroll 1
  for (int a = 0; a < SPH_NUM_ACC; ++a) {
    const SphAccel& ac = p.acc[a];
    if (ac.type == SPH_ACC_OFF) continue;
    const float3 rel = f3(__fsub_rn(xi.x, ac.pos.x), __fsub_rn(xi.y, ac.pos.y), __fsub_rn(xi.z, ac.pos.z));
    const float dt = p.timeStep;
    if (ac.type == SPH_ACC_BOX) {
      if (fabsf(rel.x) < ac.size.x && fabsf(rel.y) < ac.size.y && fabsf(rel.z) < ac.size.z) {
        add.x = __fadd_rn(add.x, __fmul_rn(ac.acc.x, dt));
        add.y = __fadd_rn(add.y, __fmul_rn(ac.acc.y, dt));
        add.z = __fadd_rn(add.z, __fmul_rn(ac.acc.z, dt));
      }
    } else if (ac.type == SPH_ACC_CYLY) {
      const float r = len2(__fdiv_rn(rel.x, ac.size.x), __fdiv_rn(rel.z, ac.size.z));
      if (fabsf(rel.y) < ac.size.y && r < 1.f) {
        add.x = __fadd_rn(add.x, __fmul_rn(ac.acc.x, dt));
        add.y = __fadd_rn(add.y, __fmul_rn(ac.acc.y, dt));
        add.z = __fadd_rn(add.z, __fmul_rn(ac.acc.z, dt));
      }
    } else if (ac.type == SPH_ACC_CYLYSM) {
      const float r = len2(rel.x, rel.z);
      if (fabsf(rel.y) < ac.size.y && r < ac.size.x) {
        const float w = __fsub_rn(1.f, __fdiv_rn(r, ac.size.z));
        add.x = __fadd_rn(add.x, __fmul_rn(__fmul_rn(ac.acc.x, w), dt));
        add.y = __fadd_rn(add.y, __fmul_rn(__fmul_rn(ac.acc.y, w), dt));
        add.z = __fadd_rn(add.z, __fmul_rn(__fmul_rn(ac.acc.z, w), dt));
      }
    }
  }
  return add;
}

__device__ __forceinline__ float dot4(float4 a, float4 b) {
  return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z)),
                   __fmul_rn(a.w, b.w));
}

// One term of the CLR_Vel trapped-air sum (System.cu:453-460): relative
// speed x (1 - cos between the normalised (4-component) velocity and position
// sums) x W(distance, 3) with W(x, h) = (1 - x)/h for x <= h.
__device__ __forceinline__ float foam_term(float4 xi, float4 vi, float4 xj, float4 vj) {
  float4 sv = make_float4(__fadd_rn(vi.x, vj.x), __fadd_rn(vi.y, vj.y), __fadd_rn(vi.z, vj.z), __fadd_rn(vi.w, vj.w));
  float4 sx = make_float4(__fadd_rn(xi.x, xj.x), __fadd_rn(xi.y, xj.y), __fadd_rn(xi.z, xj.z), __fadd_rn(xi.w, xj.w));
  const float4 dv = make_float4(__fsub_rn(vi.x, vj.x), __fsub_rn(vi.y, vj.y), __fsub_rn(vi.z, vj.z), __fsub_rn(vi.w, vj.w));
  const float4 dx = make_float4(__fsub_rn(xi.x, xj.x), __fsub_rn(xi.y, xj.y), __fsub_rn(xi.z, xj.z), __fsub_rn(xi.w, xj.w));
  const float iv = __fdiv_rn(1.0f, __fsqrt_rn(dot4(sv, sv))), ix = __fdiv_rn(1.0f, __fsqrt_rn(dot4(sx, sx)));
  sv = make_float4(__fmul_rn(sv.x, iv), __fmul_rn(sv.y, iv), __fmul_rn(sv.z, iv), __fmul_rn(sv.w, iv));
  sx = make_float4(__fmul_rn(sx.x, ix), __fmul_rn(sx.y, ix), __fmul_rn(sx.z, ix), __fmul_rn(sx.w, ix));
  const float r = __fsqrt_rn(dot4(dx, dx));
  const float w = r <= 3.0f ? __fdiv_rn(__fsub_rn(1.f, r), 3.0f) : 0.0f;
  return __fmul_rn(__fmul_rn(__fsqrt_rn(dot4(dv, dv)), __fsub_rn(1.0f, dot4(sv, sx))), w);
}

__device__ __forceinline__ float phi_clamp(float I, float tmin, float tmax) {
  return __fdiv_rn(__fsub_rn(fminf(I, tmax), fminf(I, tmin)), __fsub_rn(tmax, tmin));
}

// Colour and dye of computeForceD (System.cu:405-546); `vdiff` is the
// foam sum for CLR_Vel.  Returns false when nothing is written (CLR_None).
__device__ inline bool color_dye(const SimParams& p, float4 xi, float4 vi, float dens, float3 add,
                                 float vdiff, float* dye, float4& clr) {
  float cx = 0.2f, cy = 0.5f, cz = 1.f, intens = 0.f;
  const float dt = p.timeStep;
  switch (p.clrType) {
    case SPH_CLR_VEL: {
      const float v = __fmul_rn(2.5f, len3(f3(vi.x, vi.y, vi.z)));
      const float clrV = __fadd_rn(p.brightness, __fmul_rn(p.contrast, v));
      intens = clrV;
      const float trapped = phi_clamp(vdiff, 5.0f, 20.0f);
      const float kEnergy = __fmul_rn(__fmul_rn(__fmul_rn(p.particleMass, 1000.f), dot4(vi, vi)), 0.5f);
      const float kPot = phi_clamp(kEnergy, 0.1f, 1.0f);
      const float Nd = __fmul_rn(kPot, __fadd_rn(__fmul_rn(3.0f, trapped), __fmul_rn(3.0f, 0.0f)));
      cx = cy = cz = Nd;
    } break;
    case SPH_CLR_VELACC: {
      const float v = __fmul_rn(2.5f, len3(f3(vi.x, vi.y, vi.z)));
      const float f = __fdiv_rn(__fmul_rn(0.02f, len3(add)), dt);
      const float clrV = __fadd_rn(p.brightness, __fmul_rn(p.contrast, v));
      const float clrF = __fmul_rn(p.contrast, f);
      cx = __fadd_rn(__fmul_rn(cx, clrV), __fmul_rn(0.7f, clrF));
      cy = __fadd_rn(__fmul_rn(cy, clrV), __fmul_rn(0.35f, clrF));
      cz = __fadd_rn(__fmul_rn(cz, clrV), __fmul_rn(0.f, clrF));
    } break;
    case SPH_CLR_DENSACC: {
      const float d = __fdiv_rn(__fmul_rn(4.f, __fsub_rn(dens, p.restDensity)), p.restDensity);
      const float f = __fdiv_rn(__fmul_rn(0.02f, len3(add)), dt);
      const float clrD = __fadd_rn(p.brightness, __fmul_rn(p.contrast, d));
      const float clrF = __fmul_rn(p.contrast, f);
      cx = __fadd_rn(__fmul_rn(cx, clrD), __fmul_rn(0.7f, clrF));
      cy = __fadd_rn(__fmul_rn(cy, clrD), __fmul_rn(0.7f, clrF));
      cz = __fadd_rn(__fmul_rn(cz, clrD), __fmul_rn(0.f, clrF));
    } break;
    case SPH_CLR_VELRGB: {
      const float s = __fmul_rn(p.contrast, 2.5f);
      cx = __fadd_rn(0.5f, __fmul_rn(s, vi.x));
      cy = __fadd_rn(0.5f, __fmul_rn(s, vi.y));
      cz = __fadd_rn(0.5f, __fmul_rn(s, vi.z));
    } break;
    case SPH_CLR_ACCEL: {
      const float f = __fdiv_rn(__fmul_rn(0.02f, len3(add)), dt);
      const float clrF = __fadd_rn(p.brightness, __fmul_rn(p.contrast, f));
      intens = clrF;
      cx = __fmul_rn(cx, clrF);
      cy = __fmul_rn(cy, clrF);
      cz = __fmul_rn(cz, clrF);
    } break;
    case SPH_CLR_DENS: {
      const float d = __fdiv_rn(__fmul_rn(4.f, __fsub_rn(dens, p.restDensity)), p.restDensity);
      const float clrD = __fadd_rn(p.brightness, __fmul_rn(p.contrast, d));
      intens = clrD;
      cx = __fmul_rn(cx, clrD);
      cy = __fmul_rn(cy, clrD);
      cz = __fmul_rn(cz, clrD);
    } break;
    default:
      return false;
  }
  if (p.iHue == 1) {
    cx = intens;
    cy = 0.f;
  }
  if (dye) {
    if (p.dyeClear > 0) {
      *dye = 0.f;
    } else if (p.dyeType > 0) {
      float dyeCl = *dye;
      const float rx = __fsub_rn(xi.x, p.dyePos.x), ry = __fsub_rn(xi.y, p.dyePos.y),
                  rz = __fsub_rn(xi.z, p.dyePos.z);
      if (p.dyeType == 1) {
        if (fabsf(rx) < p.dyeSize.x && fabsf(ry) < p.dyeSize.y && fabsf(rz) < p.dyeSize.z) dyeCl = 1.f;
      } else if (p.dyeType == 2) {
        if (len3(f3(rx, ry, rz)) < p.dyeSize.y) dyeCl = 1.f;
      }
      dyeCl = __fsub_rn(dyeCl, __fmul_rn(dt, p.dyeFade));
      if (dyeCl < 0.f) dyeCl = 0.f;
      if (dyeCl >= 0.f) *dye = dyeCl;
      if (p.iHue == 0) {
        cx = __fadd_rn(cx, __fmul_rn(0.9f, dyeCl));
        cy = __fadd_rn(cy, __fmul_rn(0.9f, dyeCl));
        cz = __fadd_rn(cz, __fmul_rn(1.f, dyeCl));
      } else {
        cy = dyeCl;
      }
    }
  }
  clr = make_float4(cx, cy, cz, 1.f);
  return true;
}

}  // namespace sph
