// Structured-brick stencil of the linear-elastic Hex8 operator: the tile code shared by
// the single-solve kernels (grid.cu) and the batched request engine (bricks.cu).
//
// Linear-elastic Hex8 residual / HVP on a structured brick: the assembled operator as
// a 27-point stencil of 3 x 3 blocks.
//
// When the mesh is a tensor grid of Nx x Ny x Nz nodes with uniform spacing (hx, hy,
// hz) along each axis, node ids i + Nx (j + Ny k) and one element per cell with the
// corner order of the reference Hexahedron8 (tatva/element/base.py:478-491), every
// element has the same stiffness matrix and the HVP y = sum_e K_e v_e is, at a node
// whose eight surrounding cells all exist, a fixed stencil.  With 1-D factors on an
// axis of spacing h
//   K(0) = 2/h, K(+-1) = -1/h          (int phi_n' phi_m')
//   M(0) = 2h/3, M(+-1) = h/6          (int phi_n phi_m)
//   G(d) = -d/2                        (int phi_n' phi_{n+d})
// the 3 x 3 block for an input node at offset d = (dx, dy, dz) is
//   C_aa(d) = mu (Kx My Mz + Mx Ky Mz + Mx My Kz)(d) + (lambda + mu) D_aa(d),
//             D_xx = Kx My Mz, D_yy = Mx Ky Mz, D_zz = Mx My Kz,
//   C_ab(d) = -(lambda + mu) G(d_a) G(d_b) M(d_c)      (a != b, c the third axis),
// i.e. mu delta_ab sum_i D_ii + lambda D_ab + mu D_ba of the energy
// 1/2 sigma:eps (tests/test_sparse_benchmark.py:30-78), integrated exactly -- the
// 2 x 2 x 2 Gauss rule of the element is exact for these products -- so the stencil
// equals the element-by-element sum up to rounding.  This is what jax.jvp(jax.grad(E))
// computes for E = integrate(psi(grad u)) (README.md:93, tatva/sparse/base.py:257-265).
//
// Schedule (one launch):
//   * interior CTAs: a tile of 32 x 8 node columns (x, y) and a run of z planes.  Each
//     thread owns one column and sweeps z; the input plane (with a one-node halo, 34 x
//     10 nodes, 3 components in a 16-byte slot) sits in shared memory; a plane adds its
//     contributions to the outputs at z - 1, z, z + 1 (three accumulator sets), so each
//     output is complete after its upper neighbour plane.  Planes arrive through
//     registers two planes ahead (the Dirichlet mask is applied on the way) and are
//     double-buffered in shared memory: one barrier per plane.  Per node and plane:
//     nine 16-byte shared loads and ~90 FP operations, using the stencil's symmetries
//     (in-plane sums grouped by |dx|, |dy| for the diagonal blocks; signed cross sums
//     for the off-diagonal ones).
//   * boundary CTAs: the nodes of the z and y faces, one per thread, as the sum over
//     the cells that exist around the node of the element matrix (24 x 24, staged in
//     shared memory) times the cell's input values; the x faces in 16 x 16 patches
//     whose two node columns next to the face are staged in shared memory first.
// Every output is written once by the thread that owns it, in a fixed order: the
// result is deterministic and needs no atomics, partial slots or second pass.
#pragma once

#include <type_traits>

#include "tg_cg.cuh"
#include "tg_common.cuh"
#include "tg_internal.h"

namespace tg {

// Tile height (node rows per CTA), CTAs per SM asked of the register allocator (FP32;
// FP64 asks for 2, its kernels being FP64-pipe bound), and interior planes per tile;
// measured on GB300 (128^3 brick).
#ifndef TG_GRID_TY
#define TG_GRID_TY 8
#endif
#ifndef TG_GRID_MINB
#define TG_GRID_MINB 3
#endif
#ifndef TG_GRID_TZ
#define TG_GRID_TZ 11
#endif
constexpr int GR_TX = 32, GR_TY = TG_GRID_TY, GR_THREADS = GR_TX * GR_TY;
constexpr int GR_PX = GR_TX + 2, GR_PY = GR_TY + 2, GR_PLANE = GR_PX * GR_PY;  // 340
constexpr int GR_SLOTS = (GR_PLANE + GR_THREADS - 1) / GR_THREADS;            // 2
constexpr int GR_BNODES = GR_THREADS;                 // z / y face nodes per CTA
constexpr int GR_XT = 16;                             // x-face patch: GR_XT x GR_XT nodes
constexpr int GR_XS = GR_XT + 2;                      // staged rows per axis (with halo)
static_assert(GR_XT * GR_XT == GR_THREADS, "one x-face node per thread");
static_assert(2 * GR_XS * GR_XS <= 2 * GR_PLANE, "x-face staging fits the plane buffers");

template <class T>
struct GridCoef {
  T c[3][8];   // diagonal blocks: c[a][ix + 2 iy + 4 iz], i* = |d*| in {0, 1}
  T qxy[2];    // -(lambda + mu)/4 M_z(0), M_z(1)
  T qxz[2];    // -(lambda + mu)/4 M_y(0), M_y(1)
  T qyz[2];    // -(lambda + mu)/4 M_x(0), M_x(1)
  T r1[3];     // in-plane row sum of the |dz| = 1 diagonal-block coefficients
  T ke[8][8][3][3];  // element matrix, corners cn, cm = lx + 2 ly + 4 lz
  int nx, ny, nz;    // nodes per axis
  int tiles_x, tiles_y, tiles_z, tz;  // interior tiling: tz planes per tile
  int n_boundary_ctas;   // z and y face nodes, one per thread
  int xt_y, xt_z;        // x-face patches per face along y and z
  int n_xface_ctas;      // 2 xt_y xt_z
  int64_t n_boundary;    // z and y face nodes
};

template <class T>
struct Vec4;
template <>
struct Vec4<float> {
  using type = float4;
};
template <>
struct Vec4<double> {
  using type = double4;
};

template <class T>
__device__ __forceinline__ typename Vec4<T>::type make4(T a, T b, T c) {
  typename Vec4<T>::type r;
  r.x = a;
  r.y = b;
  r.z = c;
  r.w = T(0);
  return r;
}

// Dirichlet masks: none, one byte per dof (the C ABI's `fixed`), or one byte per node
// with bit d set when dof 3 n + d is fixed (packed once per solve by the CG, so that a
// node's mask is one load instead of three)
// MASK_NODE_OUT: the node byte applied to the output rows only -- for inputs that are
// already zero on the fixed dofs (the CG's direction when the preconditioner is zero
// there), so the staged loads need no mask.
constexpr int MASK_NONE = 0, MASK_DOF = 1, MASK_NODE = 2, MASK_NODE_OUT = 3;

// whether the launch masks its input values (the Dirichlet columns of an HVP)
template <int MODE, int MK>
__device__ __forceinline__ constexpr bool masks_input() {
  return MODE == TG_MODE_HVP && MK != MASK_NONE && MK != MASK_NODE_OUT;
}

// p.q (or r.r) of a grid launch: per node the three products summed in T (FMAs), the
// node sums accumulated in FP64, in a fixed order -- a few instructions per node where
// the compensated float pair of the vector kernels costs about thirty.
template <class T>
struct GridDotAcc {
  double v = 0.0;
  __device__ __forceinline__ void add3(const T (&a)[3], const T (&b)[3]) {
    v += (double)fma(a[2], b[2], fma(a[1], b[1], a[0] * b[0]));
  }
  __device__ __forceinline__ double value() const { return v; }
};

// Output of a launch: the operator applied (EPI_PLAIN; with DOT, p.q of input and
// output), or the residual y = b - A x of a right-hand side b (EPI_RESID; with DOT,
// y.y).
constexpr int EPI_PLAIN = 0, EPI_RESID = 1;

// bit d of the mask of node g (0: free)
template <int MK>
__device__ __forceinline__ int mask_bits(const uint8_t* __restrict__ fixed, int64_t g) {
  if constexpr (MK == MASK_DOF) {
    return (__ldg(fixed + 3 * g) != 0) | (__ldg(fixed + 3 * g + 1) != 0) << 1 |
           (__ldg(fixed + 3 * g + 2) != 0) << 2;
  } else if constexpr (MK == MASK_NODE || MK == MASK_NODE_OUT) {
    return __ldg(fixed + g);
  } else {
    return 0;
  }
}

// One input plane's contributions to the outputs below (accM, z - 1), at (accP, z) and
// above (accN, z + 1) the plane, for the node column at shared-memory slot c0.
//
// Difference form (FP32): every block row of the stencil sums to zero (a rigid
// translation has no stiffness), so each in-plane neighbour enters as its difference
// to the column's value in that plane, and the column's own values enter as the
// second difference along z with the in-plane row sum R1 of the |dz| = 1
// coefficients.  For smooth fields this keeps the FP32 result as accurate as its
// rounded input allows (the value form loses a factor of ~1/h^2 to cancellation).
// FP64 uses the value form (fewer operations on the FP64 pipe, no precision to win).
// prev: the column's value in the previous plane (difference form, updated here);
// ctr: this plane's column value (out).
template <class T>
__device__ __forceinline__ void stencil_plane(const GridCoef<T>& P,
                                              const typename Vec4<T>::type* buf, int c0,
                                              T (&accM)[3], T (&accP)[3], T (&accN)[3],
                                              T (&prev)[3], T (&ctr)[3]) {
  using V4 = typename Vec4<T>::type;
  constexpr bool DIFF = std::is_same<T, float>::value;
  // the nine in-plane neighbours, v[dy + 1][dx + 1]
  V4 v[3][3];
#pragma unroll
  for (int dy = 0; dy < 3; ++dy)
#pragma unroll
    for (int dx = 0; dx < 3; ++dx) v[dy][dx] = buf[c0 + (dx - 1) + GR_PX * (dy - 1)];
  const T a0[3] = {v[1][1].x, v[1][1].y, v[1][1].z};
  const T xm[3] = {v[1][0].x, v[1][0].y, v[1][0].z}, xp[3] = {v[1][2].x, v[1][2].y, v[1][2].z};
  const T ym[3] = {v[0][1].x, v[0][1].y, v[0][1].z}, yp[3] = {v[2][1].x, v[2][1].y, v[2][1].z};
  const T mm[3] = {v[0][0].x, v[0][0].y, v[0][0].z}, pm[3] = {v[0][2].x, v[0][2].y, v[0][2].z};
  const T mp[3] = {v[2][0].x, v[2][0].y, v[2][0].z}, pp[3] = {v[2][2].x, v[2][2].y, v[2][2].z};
  // diagonal blocks grouped by |dx|, |dy|
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    ctr[a] = a0[a];
    if constexpr (DIFF) {
      const T gx = (xm[a] - a0[a]) + (xp[a] - a0[a]);
      const T gy = (ym[a] - a0[a]) + (yp[a] - a0[a]);
      const T gc = ((mm[a] - a0[a]) + (mp[a] - a0[a])) + ((pm[a] - a0[a]) + (pp[a] - a0[a]));
      const T s0 = fma(P.c[a][3], gc, fma(P.c[a][2], gy, P.c[a][1] * gx));
      const T s1 = fma(P.c[a][7], gc, fma(P.c[a][6], gy, P.c[a][5] * gx));
      const T dz = a0[a] - prev[a];
      accP[a] = fma(-P.r1[a], dz, accP[a] + s0);
      accM[a] = fma(P.r1[a], dz, accM[a] + s1);
      accN[a] += s1;
      prev[a] = a0[a];
    } else {
      const T gx = xm[a] + xp[a], gy = ym[a] + yp[a];
      const T gc = (mm[a] + mp[a]) + (pm[a] + pp[a]);
      accP[a] = fma(P.c[a][3], gc, fma(P.c[a][2], gy, fma(P.c[a][1], gx, fma(P.c[a][0], a0[a], accP[a]))));
      const T s1 = fma(P.c[a][7], gc, fma(P.c[a][6], gy, fma(P.c[a][5], gx, P.c[a][4] * a0[a])));
      accM[a] += s1;
      accN[a] += s1;
    }
  }
  // x-y blocks: C = qxy(|dz|) dx dy, the cross sum of the in-plane corners
  const T wx = (pp[0] - pm[0]) - (mp[0] - mm[0]);
  const T wy = (pp[1] - pm[1]) - (mp[1] - mm[1]);
  accP[0] = fma(P.qxy[0], wy, accP[0]);
  accM[0] = fma(P.qxy[1], wy, accM[0]);
  accN[0] = fma(P.qxy[1], wy, accN[0]);
  accP[1] = fma(P.qxy[0], wx, accP[1]);
  accM[1] = fma(P.qxy[1], wx, accM[1]);
  accN[1] = fma(P.qxy[1], wx, accN[1]);
  // x-z blocks: C = qxz(|dy|) dx dz: odd in x, summed over dy with M_y
  const T uz_x = fma(P.qxz[1], ((pm[2] - mm[2]) + (pp[2] - mp[2])), P.qxz[0] * (xp[2] - xm[2]));
  const T ux_x = fma(P.qxz[1], ((pm[0] - mm[0]) + (pp[0] - mp[0])), P.qxz[0] * (xp[0] - xm[0]));
  // y-z blocks: C = qyz(|dx|) dy dz: odd in y, summed over dx with M_x
  const T uz_y = fma(P.qyz[1], ((mp[2] - mm[2]) + (pp[2] - pm[2])), P.qyz[0] * (yp[2] - ym[2]));
  const T uy_y = fma(P.qyz[1], ((mp[1] - mm[1]) + (pp[1] - pm[1])), P.qyz[0] * (yp[1] - ym[1]));
  // dz = plane - output: the output below (z - 1) sees dz = +1, the one above -1
  accM[0] += uz_x;
  accN[0] -= uz_x;
  accM[2] += ux_x;
  accN[2] -= ux_x;
  accM[1] += uz_y;
  accN[1] -= uz_y;
  accM[2] += uy_y;
  accN[2] -= uy_y;
}

// Interior tile: thread (lx, ly) owns node column (x0 + lx, y0 + ly), planes
// [zs, ze) of output.
template <class T, int MODE, int MK, bool DOT, int EPI = EPI_PLAIN>
__device__ void grid_interior(const GridCoef<T>& P, int item, const T* __restrict__ in,
                              const T* __restrict__ vin, const uint8_t* __restrict__ fixed,
                              T* __restrict__ y, typename Vec4<T>::type* sm, GridDotAcc<T>& dot,
                              const T* __restrict__ bres = nullptr) {
  using V4 = typename Vec4<T>::type;
  const int tid = threadIdx.x;
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  const int tx = item % P.tiles_x;
  const int rest = item / P.tiles_x;
  const int ty = rest % P.tiles_y;
  const int tzi = rest / P.tiles_y;
  const int x0 = 1 + tx * GR_TX, y0 = 1 + ty * GR_TY;
  const int zs = 1 + tzi * P.tz;
  const int ze = min(zs + P.tz, nz - 1);
  const int lx = tid % GR_TX, ly = tid / GR_TX;
  const int x = x0 + lx, yy = y0 + ly;
  const bool own = (x <= nx - 2) && (yy <= ny - 2);
  const int64_t plane_nodes = (int64_t)nx * ny;

  // staged slots of this thread: s = tid + k * GR_THREADS < GR_PLANE
  int64_t soff[GR_SLOTS];  // node offset within a plane, -1: outside the grid / no slot
#pragma unroll
  for (int k = 0; k < GR_SLOTS; ++k) {
    const int s = tid + k * GR_THREADS;
    soff[k] = -1;
    if (s < GR_PLANE) {
      const int gx = x0 - 1 + s % GR_PX, gy = y0 - 1 + s / GR_PX;
      if (gx < nx && gy < ny) soff[k] = gx + (int64_t)nx * gy;
    }
  }
  // raw values and mask bits stay in registers until the plane is stored, so that no
  // load is waited for before then (the prefetch distance is two planes)
  auto load_plane = [&](int p, T (&r)[GR_SLOTS][3], int (&m)[GR_SLOTS]) {
#pragma unroll
    for (int k = 0; k < GR_SLOTS; ++k) {
      m[k] = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) r[k][d] = T(0);
      if (soff[k] >= 0 && p <= ze) {
        const int64_t g = soff[k] + plane_nodes * p;
        if (masks_input<MODE, MK>()) m[k] = mask_bits<MK>(fixed, g);
#pragma unroll
        for (int d = 0; d < 3; ++d) r[k][d] = __ldg(in + 3 * g + d);
      }
    }
  };
  auto store_plane = [&](V4* buf, const T (&r)[GR_SLOTS][3], const int (&m)[GR_SLOTS]) {
#pragma unroll
    for (int k = 0; k < GR_SLOTS; ++k) {
      const int s = tid + k * GR_THREADS;
      if (s < GR_PLANE)
        buf[s] = make4<T>((m[k] & 1) ? T(0) : r[k][0], (m[k] & 2) ? T(0) : r[k][1],
                          (m[k] & 4) ? T(0) : r[k][2]);
    }
  };

  T accM[3], accP[3], accN[3];  // outputs at z - 1, z, z + 1 of the current plane z
#pragma unroll
  for (int a = 0; a < 3; ++a) accM[a] = accP[a] = accN[a] = T(0);
  const int c0 = (lx + 1) + GR_PX * (ly + 1);

  T prev[3], ctr[3];  // the column's value in the previous / current plane
  auto plane_step = [&](const V4* buf) { stencil_plane<T>(P, buf, c0, accM, accP, accN, prev, ctr); };

  // pc: the node's own input (the column's value in the output plane, masked): with
  // DOT the product input . output of the owned dofs (fixed dofs: their unmasked input,
  // which is also their output) enters the CTA's dot partial
  // the output node's mask bits, loaded one plane before its emission
  auto out_mask = [&](int z) {
    return (own && z >= zs && z < ze) ? mask_bits<MK>(fixed, x + (int64_t)nx * yy + plane_nodes * z)
                                      : 0;
  };
  auto emit = [&](int z, const T (&acc)[3], const T (&pc)[3], int m) {
    if (!own || z < zs || z >= ze) return;
    const int64_t g = x + (int64_t)nx * yy + plane_nodes * z, base = 3 * g;
    T pvs[3], vals[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      T val = acc[d], pv = pc[d];
      if (m >> d & 1) {
        val = (MODE == TG_MODE_HVP) ? __ldg(vin + base + d) : T(0);
        pv = val;
      }
      if constexpr (EPI == EPI_RESID) {
        val = __ldg(bres + base + d) - val;
        pv = val;
      }
      y[base + d] = val;
      pvs[d] = pv;
      vals[d] = val;
    }
    if constexpr (DOT) dot.add3(pvs, vals);
  };

  V4* buf0 = sm;
  V4* buf1 = sm + GR_PLANE;
  T rA[GR_SLOTS][3], rB[GR_SLOTS][3];
  int mA[GR_SLOTS], mB[GR_SLOTS];
  // prologue: plane zs - 1 into buf0; zs in flight in rB, zs + 1 in rA
  load_plane(zs - 1, rA, mA);
  store_plane(buf0, rA, mA);
  load_plane(zs, rB, mB);
  load_plane(zs + 1, rA, mA);
  int m_out = out_mask(zs - 1);  // mask of the node emitted after the next plane
  __syncthreads();
  {  // the first plane's step then sees no z difference (its outputs are discarded)
    const V4 c = buf0[c0];
    prev[0] = c.x;
    prev[1] = c.y;
    prev[2] = c.z;
  }
  // planes p = zs - 1 .. ze, two per trip: buf0 holds p, buf1 gets p + 1
  ctr[0] = ctr[1] = ctr[2] = T(0);
  for (int p = zs - 1; p <= ze; p += 2) {
    T pc[3] = {ctr[0], ctr[1], ctr[2]};
    int m_now = m_out;
    m_out = out_mask(p);
    plane_step(buf0);
    emit(p - 1, accM, pc, m_now);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      accM[a] = accP[a];
      accP[a] = accN[a];
      accN[a] = T(0);
    }
    store_plane(buf1, rB, mB);
    load_plane(p + 3, rB, mB);
    __syncthreads();
    if (p + 1 > ze) break;
#pragma unroll
    for (int a = 0; a < 3; ++a) pc[a] = ctr[a];
    m_now = m_out;
    m_out = out_mask(p + 1);
    plane_step(buf1);
    emit(p, accM, pc, m_now);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      accM[a] = accP[a];
      accP[a] = accN[a];
      accN[a] = T(0);
    }
    store_plane(buf0, rA, mA);
    load_plane(p + 4, rA, mA);
    __syncthreads();
  }
}

// Boundary node t of the six faces: z = 0 and z = nz - 1 (all nx ny nodes), y = 0 and
// y = ny - 1 (nx (nz - 2)), x = 0 and x = nx - 1 ((ny - 2)(nz - 2)).
__device__ __forceinline__ void boundary_node(int64_t t, int nx, int ny, int nz, int& x, int& y,
                                              int& z) {
  const int64_t fz = (int64_t)nx * ny, fy = (int64_t)nx * (nz - 2);
  if (t < 2 * fz) {
    z = t < fz ? 0 : nz - 1;
    const int64_t r = t < fz ? t : t - fz;
    x = (int)(r % nx);
    y = (int)(r / nx);
    return;
  }
  t -= 2 * fz;
  if (t < 2 * fy) {
    y = t < fy ? 0 : ny - 1;
    const int64_t r = t < fy ? t : t - fy;
    x = (int)(r % nx);
    z = 1 + (int)(r / nx);
    return;
  }
  t -= 2 * fy;
  const int64_t fx = (int64_t)(ny - 2) * (nz - 2);
  x = t < fx ? 0 : nx - 1;
  const int64_t r = t < fx ? t : t - fx;
  y = 1 + (int)(r % (ny - 2));
  z = 1 + (int)(r / (ny - 2));
}

// Output of a face node: the Dirichlet rows, the residual epilogue and the dot.
template <class T, int MODE, int MK, bool DOT, int EPI>
__device__ __forceinline__ void grid_emit_node(int x, int yy, int z, int nx, int ny,
                                               const T (&acc)[3], const T* __restrict__ in,
                                               const T* __restrict__ vin,
                                               const uint8_t* __restrict__ fixed,
                                               T* __restrict__ y, GridDotAcc<T>& dot,
                                               const T* __restrict__ bres) {
  const int64_t gn = x + (int64_t)nx * (yy + (int64_t)ny * z), base = 3 * gn;
  const int mn = mask_bits<MK>(fixed, gn);
  T pvs[3], vals[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    T val = acc[d];
    T pv = T(0);
    if constexpr (DOT && EPI == EPI_PLAIN) pv = __ldg(in + base + d);
    if (mn >> d & 1) {
      val = (MODE == TG_MODE_HVP) ? __ldg(vin + base + d) : T(0);
      pv = val;
    }
    if constexpr (EPI == EPI_RESID) {
      val = __ldg(bres + base + d) - val;
      pv = val;
    }
    y[base + d] = val;
    pvs[d] = pv;
    vals[d] = val;
  }
  if constexpr (DOT) dot.add3(pvs, vals);
}

// Nodes of the z and y faces, one per thread: the sum over the cells that exist
// around the node of the element matrix times the cell's input values.  Consecutive
// threads are consecutive along x, so the corner loads coalesce.
template <class T, int MODE, int MK, bool DOT, int EPI = EPI_PLAIN>
__device__ void grid_boundary(const GridCoef<T>& P, int64_t t0, const T* __restrict__ in,
                              const T* __restrict__ vin, const uint8_t* __restrict__ fixed,
                              T* __restrict__ y, T* ke, GridDotAcc<T>& dot,
                              const T* __restrict__ bres = nullptr) {
  for (int i = threadIdx.x; i < 8 * 8 * 9; i += blockDim.x) ke[i] = (&P.ke[0][0][0][0])[i];
  __syncthreads();
  const int64_t t = t0 + threadIdx.x;
  if (t >= P.n_boundary) return;
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  int x, yy, z;
  boundary_node(t, nx, ny, nz, x, yy, z);
  T acc[3] = {T(0), T(0), T(0)};
  for (int o = 0; o < 8; ++o) {  // cell whose corner o is this node
    const int cx = x - (o & 1), cy = yy - ((o >> 1) & 1), cz = z - (o >> 2);
    if (cx < 0 || cy < 0 || cz < 0 || cx >= nx - 1 || cy >= ny - 1 || cz >= nz - 1) continue;
    const T* kr = ke + o * 72;  // rows of corner o: [cm][a][b]
#pragma unroll
    for (int cm = 0; cm < 8; ++cm) {
      const int64_t g = (cx + (cm & 1)) + (int64_t)nx * ((cy + ((cm >> 1) & 1)) +
                                                         (int64_t)ny * (cz + (cm >> 2)));
      const int m = masks_input<MODE, MK>() ? mask_bits<MK>(fixed, g) : 0;
      const T v0 = (m & 1) ? T(0) : __ldg(in + 3 * g);
      const T v1 = (m & 2) ? T(0) : __ldg(in + 3 * g + 1);
      const T v2 = (m & 4) ? T(0) : __ldg(in + 3 * g + 2);
      const T* k9 = kr + cm * 9;
#pragma unroll
      for (int a = 0; a < 3; ++a) acc[a] = fma(k9[3 * a + 2], v2, fma(k9[3 * a + 1], v1, fma(k9[3 * a], v0, acc[a])));
    }
  }
  grid_emit_node<T, MODE, MK, DOT, EPI>(x, yy, z, nx, ny, acc, in, vin, fixed, y, dot, bres);
}

// Nodes of the two x faces (x = 0 and x = nx - 1, 1 <= y <= ny - 2, 1 <= z <= nz - 2),
// a GR_XT x GR_XT patch (y, z) per CTA.  On these faces consecutive nodes are a grid
// row apart, so per-thread corner loads would touch one cache line per thread; the CTA
// instead stages the two node columns next to the face (x = 0, 1 or nx - 2, nx - 1)
// of its patch and halo, row by row (contiguous 24-byte runs), masked on the way.
// All four cells around such a node exist, so the element-matrix indices are
// compile-time constants.
template <class T, int MODE, int MK, bool DOT, int EPI = EPI_PLAIN>
__device__ void grid_xface(const GridCoef<T>& P, int item, const T* __restrict__ in,
                           const T* __restrict__ vin, const uint8_t* __restrict__ fixed,
                           T* __restrict__ y, typename Vec4<T>::type* sm, GridDotAcc<T>& dot,
                           const T* __restrict__ bres = nullptr) {
  using V4 = typename Vec4<T>::type;
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  const int per_face = P.xt_y * P.xt_z;
  const int face = item / per_face, rest = item - face * per_face;
  const int ty = rest % P.xt_y, tz = rest / P.xt_y;
  const int xb = face ? nx - 2 : 0;  // first of the two staged columns
  const int y0 = 1 + ty * GR_XT, z0 = 1 + tz * GR_XT;
  // slot s = 2 (rz GR_XS + ry) + col: node (xb + col, y0 - 1 + ry, z0 - 1 + rz)
  for (int s = threadIdx.x; s < 2 * GR_XS * GR_XS; s += blockDim.x) {
    const int col = s & 1, r = s >> 1;
    const int gy = y0 - 1 + r % GR_XS, gz = z0 - 1 + r / GR_XS;
    T v0 = T(0), v1 = T(0), v2 = T(0);
    if (gy < ny && gz < nz) {
      const int64_t g = (xb + col) + (int64_t)nx * (gy + (int64_t)ny * gz);
      const int m = masks_input<MODE, MK>() ? mask_bits<MK>(fixed, g) : 0;
      v0 = (m & 1) ? T(0) : __ldg(in + 3 * g);
      v1 = (m & 2) ? T(0) : __ldg(in + 3 * g + 1);
      v2 = (m & 4) ? T(0) : __ldg(in + 3 * g + 2);
    }
    sm[s] = make4<T>(v0, v1, v2);
  }
  __syncthreads();
  const int ly = threadIdx.x % GR_XT, lz = threadIdx.x / GR_XT;
  const int yy = y0 + ly, z = z0 + lz;
  if (yy > ny - 2 || z > nz - 2) return;
  T acc[3] = {T(0), T(0), T(0)};
  auto cells = [&](auto ox_c) {
    constexpr int OX = decltype(ox_c)::value;  // the node is corner x-index OX of its cells
#pragma unroll
    for (int oyz = 0; oyz < 4; ++oyz) {
      const int oy = oyz & 1, oz = oyz >> 1;
      const int o = OX + 2 * oy + 4 * oz;
#pragma unroll
      for (int cm = 0; cm < 8; ++cm) {
        const int cmx = cm & 1, cmy = (cm >> 1) & 1, cmz = cm >> 2;
        const V4 v = sm[2 * ((lz + 1 - oz + cmz) * GR_XS + (ly + 1 - oy + cmy)) + cmx];
#pragma unroll
        for (int a = 0; a < 3; ++a)
          acc[a] = fma(P.ke[o][cm][a][2], v.z, fma(P.ke[o][cm][a][1], v.y, fma(P.ke[o][cm][a][0], v.x, acc[a])));
      }
    }
  };
  if (face) cells(std::integral_constant<int, 1>{});
  else cells(std::integral_constant<int, 0>{});
  grid_emit_node<T, MODE, MK, DOT, EPI>(face ? nx - 1 : 0, yy, z, nx, ny, acc, in, vin, fixed, y,
                                        dot, bres);
}


// ------------------------------------------------------------------------- host
// Stencil coefficients and the element matrix from the spacings and Lame parameters,
// in FP64, then rounded to T.
template <class T>
static void grid_coefficients(const double h[3], double mu, double lam, GridCoef<T>& P) {
  double K[3][2], M[3][2];
  for (int k = 0; k < 3; ++k) {
    K[k][0] = 2.0 / h[k];
    K[k][1] = -1.0 / h[k];
    M[k][0] = 2.0 * h[k] / 3.0;
    M[k][1] = h[k] / 6.0;
  }
  for (int i = 0; i < 8; ++i) {
    const int ix = i & 1, iy = (i >> 1) & 1, iz = i >> 2;
    const double D[3] = {K[0][ix] * M[1][iy] * M[2][iz], M[0][ix] * K[1][iy] * M[2][iz],
                         M[0][ix] * M[1][iy] * K[2][iz]};
    const double L = D[0] + D[1] + D[2];
    for (int a = 0; a < 3; ++a) P.c[a][i] = (T)(mu * L + (lam + mu) * D[a]);
  }
  for (int a = 0; a < 3; ++a) {
    double r = 0.0;  // sum over dx, dy of c(dx, dy, 1): weights 1, 2, 2, 4 by class
    for (int i = 4; i < 8; ++i) {
      const int ix = i & 1, iy = (i >> 1) & 1;
      const double D[3] = {K[0][ix] * M[1][iy] * M[2][1], M[0][ix] * K[1][iy] * M[2][1],
                           M[0][ix] * M[1][iy] * K[2][1]};
      r += (ix ? 2.0 : 1.0) * (iy ? 2.0 : 1.0) * (mu * (D[0] + D[1] + D[2]) + (lam + mu) * D[a]);
    }
    P.r1[a] = (T)r;
  }
  const double q = -(lam + mu) / 4.0;
  for (int s = 0; s < 2; ++s) {
    P.qxy[s] = (T)(q * M[2][s]);
    P.qxz[s] = (T)(q * M[1][s]);
    P.qyz[s] = (T)(q * M[0][s]);
  }
  // element matrix of one cell: corners cn, cm = lx + 2 ly + 4 lz; per axis the
  // element-level 1-D integrals Kel = [[1,-1],[-1,1]]/h, Mel = h[[1/3,1/6],[1/6,1/3]],
  // Gel(A, B) = int phi_A' phi_B = s_A / 2 (s = -1 at the lower corner, +1 upper)
  for (int cn = 0; cn < 8; ++cn)
    for (int cm = 0; cm < 8; ++cm) {
      int ln[3], lm[3];
      for (int k = 0; k < 3; ++k) {
        ln[k] = (cn >> k) & 1;
        lm[k] = (cm >> k) & 1;
      }
      auto DE = [&](int i, int j) {
        double v = 1.0;
        for (int k = 0; k < 3; ++k) {
          double f;
          if (i == j && j == k) f = (ln[k] == lm[k] ? 1.0 : -1.0) / h[k];
          else if (k == i) f = (ln[k] ? 0.5 : -0.5);
          else if (k == j) f = (lm[k] ? 0.5 : -0.5);
          else f = h[k] * (ln[k] == lm[k] ? 1.0 / 3.0 : 1.0 / 6.0);
          v *= f;
        }
        return v;
      };
      const double Ls = DE(0, 0) + DE(1, 1) + DE(2, 2);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          P.ke[cn][cm][a][b] = (T)(lam * DE(a, b) + mu * DE(b, a) + (a == b ? mu * Ls : 0.0));
    }
}

// SMs of the current device (queried once per device).
static int grid_sm_count() {
  static int cached[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cached[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cached[dev] = n;
  }
  return cached[dev];
}

// Coefficients and tiling of a brick of nodes[0] x nodes[1] x nodes[2] nodes with
// spacings h; returns the launch's CTA count (boundary CTAs first, then the interior
// tiles), or -1 when it does not fit an int.
// deep: always TG_GRID_TZ planes per tile (launches shared by many bricks need no
// spreading of one brick over the SMs, and deeper tiles reload fewer halo planes).
template <class T>
static int64_t grid_setup_dims(const int32_t nodes[3], const double h[3], double mu, double lam,
                               GridCoef<T>& P, bool deep = false) {
  const int nx = nodes[0], ny = nodes[1], nz = nodes[2];
  grid_coefficients<T>(h, mu, lam, P);
  P.nx = nx;
  P.ny = ny;
  P.nz = nz;
  const int ix = nx - 2, iy = ny - 2, iz = nz - 2;
  P.tiles_x = ix > 0 ? (ix + GR_TX - 1) / GR_TX : 0;
  P.tiles_y = iy > 0 ? (iy + GR_TY - 1) / GR_TY : 0;
  // planes per tile: TG_GRID_TZ on large grids; fewer on small ones, so that the
  // interior still spreads over about two CTAs per SM (a tile sweeps its planes one
  // after the other, which sets the latency of a small grid's HVP)
  P.tz = TG_GRID_TZ;
  if (!deep && iz > 0 && P.tiles_x > 0 && P.tiles_y > 0) {
    const int64_t columns = (int64_t)P.tiles_x * P.tiles_y;
    const int64_t want = 2 * (int64_t)grid_sm_count();
    const int64_t tz = (columns * iz + want - 1) / want;
    P.tz = (int)(tz < 2 ? 2 : (tz > TG_GRID_TZ ? TG_GRID_TZ : tz));
  }
  P.tiles_z = iz > 0 ? (iz + P.tz - 1) / P.tz : 0;
  const int64_t n_int = (int64_t)P.tiles_x * P.tiles_y * P.tiles_z;
  // the z and y faces (thread per node), then the x faces (patches)
  P.n_boundary = 2 * (int64_t)nx * ny + 2 * (int64_t)nx * (nz > 2 ? nz - 2 : 0);
  const int64_t n_bnd_ctas = (P.n_boundary + GR_BNODES - 1) / GR_BNODES;
  P.xt_y = iy > 0 ? (iy + GR_XT - 1) / GR_XT : 0;
  P.xt_z = iz > 0 ? (iz + GR_XT - 1) / GR_XT : 0;
  const int64_t n_x_ctas = 2 * (int64_t)P.xt_y * P.xt_z;
  if (n_int + n_bnd_ctas + n_x_ctas > 0x7fffffff) return -1;
  P.n_boundary_ctas = (int)n_bnd_ctas;
  P.n_xface_ctas = (int)n_x_ctas;
  return n_int + n_bnd_ctas + n_x_ctas;
}

// The same for a structured-brick plan (tg_grid_detect's nodes and spacings).
template <class T>
static int64_t grid_setup(const tg_block_plan* plan, double mu, double lam, GridCoef<T>& P) {
  return grid_setup_dims<T>(plan->grid_nodes, plan->grid_h, mu, lam, P);
}

}  // namespace tg
