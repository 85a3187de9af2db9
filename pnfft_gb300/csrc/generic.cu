// generic.cu -- interpolation B and spreading B^T with one thread per node
// in global memory, for any cutoff and grid (small node counts on large
// grids, grids below the tile size, cutoffs above 15).
//
// Reference: loop_over_particles_trafo / _adj (kernel/ndft-parallel.c:2703-3009)
// with the stencil loops of kernel/assign.c:478-1159.
#include <cuda_runtime.h>

#include "pg_conv.cuh"
#include "pg_kernels.h"
#include "pg_math.cuh"

namespace pg {

// ---------------------------------------------------------------------------
// generic kernels for any cutoff: one thread per node, global memory
// ---------------------------------------------------------------------------
template <typename T, int MODE>
__global__ void k_interp_generic(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0, DH = (MODE & 4) != 0;
  constexpr int NDER = DH ? 2 : (DG ? 1 : 0);
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.M) return;
  const int j = a.bin.perm[q];
  const int cut = a.w.cut;
  T ws[9 * 64];
  double dist[3];
  int u[3];
  for (int t = 0; t < 3; t++) {
    AxisPos p = axis_pos(a.x[3 * (int64_t)j + t], a.w.n[t], a.w.m, a.il);
    dist[t] = p.dist;
    u[t] = p.u;
  }
  for (int e = 0; e < 3 * cut; e++) {
    int t = e / cut, s = e - t * cut;
    T out[3] = {(T)0, (T)0, (T)0};
    window_point<T>(a.w, t, s, (T)dist[t], NDER, out);
    ws[e] = out[0];
    ws[3 * cut + e] = out[1];
    ws[6 * cut + e] = out[2];
  }
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const C *grid = (const C *)a.grid;
  T af_r = 0, af_i = 0, ag_r[3] = {0, 0, 0}, ag_i[3] = {0, 0, 0}, ah_r[6] = {0}, ah_i[6] = {0};
  for (int l0 = 0; l0 < cut; l0++) {
    int g0 = (u[0] + l0) % n0;
    for (int l1 = 0; l1 < cut; l1++) {
      int g1 = (u[1] + l1) % n1;
      const T px = ws[l0], py = ws[cut + l1], dx = ws[3 * cut + l0], dy = ws[3 * cut + cut + l1];
      const T ddx = ws[6 * cut + l0], ddy = ws[6 * cut + cut + l1];
      for (int l2 = 0; l2 < cut; l2++) {
        int g2 = (u[2] + l2) % n2;
        C g = grid[((size_t)g0 * n1 + g1) * n2 + g2];
        if (a.real_only) g.y = (T)0;
        const T pz = ws[2 * cut + l2], dz = ws[3 * cut + 2 * cut + l2], ddz = ws[6 * cut + 2 * cut + l2];
        if (DF) {
          af_r += px * py * pz * g.x;
          af_i += px * py * pz * g.y;
        }
        if (DG) {
          T w0 = dx * py * pz, w1 = px * dy * pz, w2 = px * py * dz;
          ag_r[0] += w0 * g.x;
          ag_i[0] += w0 * g.y;
          ag_r[1] += w1 * g.x;
          ag_i[1] += w1 * g.y;
          ag_r[2] += w2 * g.x;
          ag_i[2] += w2 * g.y;
        }
        if (DH) {
          T w[6] = {ddx * py * pz, dx * dy * pz, dx * py * dz, px * ddy * pz, px * dy * dz, px * py * ddz};
          for (int c = 0; c < 6; c++) {
            ah_r[c] += w[c] * g.x;
            ah_i[c] += w[c] * g.y;
          }
        }
      }
    }
  }
  const T scale = a.use_il ? (T)0.5 : (T)1;
  const int64_t ind = (int64_t)j * a.stride + a.offset;
  if (DF) {
    if (a.real_io) a.f_out[ind] += (double)(af_r * scale);
    else {
      a.f_out[2 * ind] += (double)(af_r * scale);
      a.f_out[2 * ind + 1] += (double)(af_i * scale);
    }
  }
  if (DG)
    for (int c = 0; c < 3; c++) {
      if (a.real_io) a.grad_out[3 * ind + c] += (double)(ag_r[c] * scale);
      else {
        a.grad_out[2 * (3 * ind + c)] += (double)(ag_r[c] * scale);
        a.grad_out[2 * (3 * ind + c) + 1] += (double)(ag_i[c] * scale);
      }
    }
  if (DH)
    for (int c = 0; c < 6; c++) {
      if (a.real_io) a.hess_out[6 * ind + c] += (double)(ah_r[c] * scale);
      else {
        a.hess_out[2 * (6 * ind + c)] += (double)(ah_r[c] * scale);
        a.hess_out[2 * (6 * ind + c) + 1] += (double)(ah_i[c] * scale);
      }
    }
}

template <typename T, int MODE>
__global__ void k_spread_generic(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0;
  constexpr int NDER = DG ? 1 : 0;
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.M) return;
  const int j = a.bin.perm[q];
  const int cut = a.w.cut;
  T ws[6 * 64];
  double dist[3];
  int u[3];
  for (int t = 0; t < 3; t++) {
    AxisPos p = axis_pos(a.x[3 * (int64_t)j + t], a.w.n[t], a.w.m, a.il);
    dist[t] = p.dist;
    u[t] = p.u;
  }
  for (int e = 0; e < 3 * cut; e++) {
    int t = e / cut, s = e - t * cut;
    T out[3] = {(T)0, (T)0, (T)0};
    window_point<T>(a.w, t, s, (T)dist[t], NDER, out);
    ws[e] = out[0];
    ws[3 * cut + e] = out[1];
  }
  const T scale = a.use_il ? (T)0.5 : (T)1;
  const int64_t ind = (int64_t)j * a.stride + a.offset;
  T f_r = 0, f_i = 0, g_r[3] = {0, 0, 0}, g_i[3] = {0, 0, 0};
  if (DF) {
    if (a.real_io) f_r = (T)a.f_in[ind];
    else {
      f_r = (T)a.f_in[2 * ind];
      f_i = (T)a.f_in[2 * ind + 1];
    }
  }
  if (DG)
    for (int c = 0; c < 3; c++) {
      if (a.real_io) g_r[c] = (T)a.grad_in[3 * ind + c];
      else {
        g_r[c] = (T)a.grad_in[2 * (3 * ind + c)];
        g_i[c] = (T)a.grad_in[2 * (3 * ind + c) + 1];
      }
    }
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  C *grid = (C *)a.grid;
  for (int l0 = 0; l0 < cut; l0++) {
    int g0 = (u[0] + l0) % n0;
    for (int l1 = 0; l1 < cut; l1++) {
      int g1 = (u[1] + l1) % n1;
      const T px = ws[l0], py = ws[cut + l1], dx = ws[3 * cut + l0], dy = ws[3 * cut + cut + l1];
      for (int l2 = 0; l2 < cut; l2++) {
        int g2 = (u[2] + l2) % n2;
        const T pz = ws[2 * cut + l2], dz = ws[3 * cut + 2 * cut + l2];
        C v;
        v.x = (T)0;
        v.y = (T)0;
        if (DF) {
          v.x += px * py * pz * f_r;
          v.y += px * py * pz * f_i;
        }
        if (DG) {
          T w0 = dx * py * pz, w1 = px * dy * pz, w2 = px * py * dz;
          v.x += w0 * g_r[0] + w1 * g_r[1] + w2 * g_r[2];
          v.y += w0 * g_i[0] + w1 * g_i[1] + w2 * g_i[2];
        }
        v.x *= scale;
        v.y *= scale;
        atomic_add_grid(&grid[((size_t)g0 * n1 + g1) * n2 + g2], v);
      }
    }
  }
}

void launch_interp_generic(const ConvArgs &a, int mode, bool fp32, cudaStream_t s) {
  const unsigned bl = (unsigned)((a.M + 127) / 128);
  if (fp32) {
    switch (mode) {
      case 1: k_interp_generic<float, 1><<<bl, 128, 0, s>>>(a); break;
      case 2: k_interp_generic<float, 2><<<bl, 128, 0, s>>>(a); break;
      case 3: k_interp_generic<float, 3><<<bl, 128, 0, s>>>(a); break;
      case 4: k_interp_generic<float, 4><<<bl, 128, 0, s>>>(a); break;
      default: break;
    }
  } else {
    switch (mode) {
      case 1: k_interp_generic<double, 1><<<bl, 128, 0, s>>>(a); break;
      case 2: k_interp_generic<double, 2><<<bl, 128, 0, s>>>(a); break;
      case 3: k_interp_generic<double, 3><<<bl, 128, 0, s>>>(a); break;
      case 4: k_interp_generic<double, 4><<<bl, 128, 0, s>>>(a); break;
      default: break;
    }
  }
}

void launch_spread_generic(const ConvArgs &a, int mode, bool fp32, cudaStream_t s) {
  const unsigned bl = (unsigned)((a.M + 127) / 128);
  if (fp32) {
    switch (mode) {
      case 1: k_spread_generic<float, 1><<<bl, 128, 0, s>>>(a); break;
      case 2: k_spread_generic<float, 2><<<bl, 128, 0, s>>>(a); break;
      case 3: k_spread_generic<float, 3><<<bl, 128, 0, s>>>(a); break;
      default: break;
    }
  } else {
    switch (mode) {
      case 1: k_spread_generic<double, 1><<<bl, 128, 0, s>>>(a); break;
      case 2: k_spread_generic<double, 2><<<bl, 128, 0, s>>>(a); break;
      case 3: k_spread_generic<double, 3><<<bl, 128, 0, s>>>(a); break;
      default: break;
    }
  }
}

}  // namespace pg
