// Gathered form of the energy fill (interface.hpp:49-60 layouts; the
// decomposition of network_flow_node.hpp:420-485 restated in lf_kernels.cu):
// per-node and per-edge shares as host/device functions, so that the kernels
// in lf_kernels.cu and a host check run the same code.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "lf_device.cuh"

namespace lfg {

// The decomposition of k_fill_energy gathered per node: node w (real
// coordinates a, b, c, real index r) adds its unary term, the source-side
// share of its own Kp pairwise terms (w -> w + d_e) and the target-side share
// of the terms that end at it (the table of node w - d_e, edge e).  Every output word has one
// writer, so the accumulation is a plain read-modify-write, and the integer
// sums equal the scattered ones exactly.
template <bool VEC>
__host__ __device__ __forceinline__ void fill_table(const int64_t* binary, int Kp, long long node,
                                                    int e, long long& A, long long& B,
                                                    long long& C, long long& D) {
  const int64_t* q = binary + (node * Kp + e) * 4;
  if (VEC) {
    const longlong2 q0 = reinterpret_cast<const longlong2*>(q)[0];
    const longlong2 q1 = reinterpret_cast<const longlong2*>(q)[1];
    A = q0.x; B = q0.y; C = q1.x; D = q1.y;
  } else {
    A = q[0]; B = q[1]; C = q[2]; D = q[3];
  }
}

// Unary share of node r: returns E0 - E1 and adds E0 to *c0.
template <bool VEC>
__host__ __device__ __forceinline__ long long fill_gather_unary(const int64_t* unary, long long r,
                                                               long long* c0) {
  long long E0, E1;
  if (VEC) {
    const longlong2 ue = reinterpret_cast<const longlong2*>(unary)[r];
    E0 = ue.x;
    E1 = ue.y;
  } else {
    E0 = unary[2 * r];
    E1 = unary[2 * r + 1];
  }
  *c0 += E0;
  return E0 - E1;
}

// Edge-e share of node w (padded index): both ends' terms of direction e,
// the capacity words of planes e and rev[e] at w (read-modify-write), the
// own term's constant added to *c0.  Returns the excess share; *bad is set
// for a non-submodular own term.
template <bool VEC>
__host__ __device__ __forceinline__ long long fill_gather_edge(
    const Geo& g, const Stencil& st, long long r, int a, int b, int c, long long w, int e,
    const int64_t* binary, long long* cap, bool* bad, long long* c0) {
  const int Kp = st.K / 2;
  const int da = st.da[e], db = st.db[e], dc = st.dc[e];
  long long x = 0, A, B, C, D;
  if (a + da >= 0 && a + da < g.A && b + db >= 0 && b + db < g.B && c + dc >= 0 &&
      c + dc < g.C) {  // own term, w is its source end
    fill_table<VEC>(binary, Kp, r, e, A, B, C, D);
    *c0 += A;
    const long long Bq = B - A, Cq = C - D;
    if (Bq + Cq < 0) *bad = true;
    long long cu = 0;
    x += A - D;
    if (Bq < 0) { x += Bq; cu = Bq + Cq; }
    else if (Cq < 0) x -= Cq;
    else cu = Cq;
    if (cu) cap[(long long)e * g.NP + w] += cu;
  }
  const int sa = a - da, sb = b - db, sc = c - dc;
  if (sa >= 0 && sa < g.A && sb >= 0 && sb < g.B && sc >= 0 && sc < g.C) {  // w is the target
    fill_table<VEC>(binary, Kp, ((long long)sa * g.B + sb) * g.C + sc, e, A, B, C, D);
    const long long Bq = B - A, Cq = C - D;
    long long cv = 0;
    if (Bq < 0) x -= Bq;
    else if (Cq < 0) { x += Cq; cv = Bq + Cq; }
    else cv = Bq;
    if (cv) cap[(long long)st.rev[e] * g.NP + w] += cv;
  }
  return x;
}

// All of node r: returns its share of the constant term.
template <bool VEC>
__host__ __device__ __forceinline__ long long fill_gather_node(
    const Geo& g, const Stencil& st, long long r, int a, int b, int c, const int64_t* unary,
    const int64_t* binary, long long* exc, long long* cap, bool* bad) {
  const long long w = ((long long)a * g.Bp + b) * g.Cp + c;
  long long c0 = 0;
  long long x = fill_gather_unary<VEC>(unary, r, &c0);
  for (int e = 0; e < st.K / 2; ++e)
    x += fill_gather_edge<VEC>(g, st, r, a, b, c, w, e, binary, cap, bad, &c0);
  if (x) exc[w] += x;
  return c0;
}

}  // namespace lfg
