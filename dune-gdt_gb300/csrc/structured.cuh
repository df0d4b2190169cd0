// Structured-grid topology shared by the pattern, assembly and adjoint kernels.
//
// Reference conventions restated (paths in the dune-gdt tree): elements and vertices of cube grids
// are lexicographic with x fastest (YaspGrid via make_cube_grid, examples/stationary-heat-equation.cc:87);
// simplex grids split every cube into d! simplices, one per axis permutation pi in
// std::next_permutation order, with corners 0, e_pi0, e_pi0 + e_pi1, ... (dune-grid's structured
// simplex factory); reference-element vertex i of a cube sits at the bits of i; simplex face f is
// opposite vertex dim - f. The continuous P1/Q1 DoF of a local vertex is the grid vertex index
// (ContinuousMapper, spaces/mapper/continuous.hh:139-150); DG DoFs are e * local_size + i
// (DiscontinuousMapper, spaces/mapper/discontinuous.hh:102-125).
#pragma once
#include "internal.cuh"

namespace gdt {

// axis moved by step m of Kuhn simplex t (permutations in lexicographic order)
__host__ __device__ constexpr int kuhn_axis(int dim, int t, int m) {
  return dim == 2 ? ((t == 0) ? m : 1 - m)
                  : (t == 0 ? (m == 0 ? 0 : m == 1 ? 1 : 2)
                     : t == 1 ? (m == 0 ? 0 : m == 1 ? 2 : 1)
                     : t == 2 ? (m == 0 ? 1 : m == 1 ? 0 : 2)
                     : t == 3 ? (m == 0 ? 1 : m == 1 ? 2 : 0)
                     : t == 4 ? (m == 0 ? 2 : m == 1 ? 0 : 1)
                              : (m == 0 ? 2 : m == 1 ? 1 : 0));
}

// cube corner (bit pattern) of local vertex j of element type t
__host__ __device__ constexpr int local_corner(int dim, bool simplex, int t, int j) {
  if (!simplex) return j;
  int c = 0;
  for (int m = 0; m < j; ++m) c |= 1 << kuhn_axis(dim, t, m);
  return c;
}

__host__ __device__ constexpr int num_sub(int dim, bool simplex) { return simplex ? (dim == 2 ? 2 : 6) : 1; }
__host__ __device__ constexpr int num_local(int dim, bool simplex) { return simplex ? dim + 1 : (1 << dim); }
__host__ __device__ constexpr int pow3(int d) { return d == 1 ? 3 : d == 2 ? 9 : 27; }

// stencil slot k in [0, 3^d): offset component a < d is (k / 3^a) % 3 - 1; ascending k is ascending
// linear vertex offset, i.e. the sorted column order of a row
__host__ __device__ constexpr int slot_offset(int k, int a) { return (a == 0 ? k : a == 1 ? k / 3 : k / 9) % 3 - 1; }
// slot of the offset between two cube corners (bit patterns) c1 - c0
__host__ __device__ constexpr int slot_between(int dim, int c0, int c1) {
  int k = 0, p = 1;
  for (int a = 0; a < dim; ++a) {
    k += (((c1 >> a) & 1) - ((c0 >> a) & 1) + 1) * p;
    p *= 3;
  }
  return k;
}
__host__ __device__ constexpr int center_slot(int dim) { return dim == 1 ? 1 : dim == 2 ? 4 : 13; }

// is slot k an edge (or the vertex itself) of the P1/Q1 vertex stencil?
__host__ __device__ constexpr bool slot_in_stencil(int dim, bool simplex, int k) {
  bool pos = true, neg = true;
  for (int a = 0; a < dim; ++a) {
    int o = slot_offset(k, a);
    if (o < 0) pos = false;
    if (o > 0) neg = false;
  }
  return simplex ? (pos || neg) : true;
}

// DG neighbours of element e, sorted by element index, self included; returns count.
// Cube grids: across the 2d faces; Kuhn triangles: A=(0,e0,e0+e1) and B=(0,e1,e0+e1) per cube.
__host__ __device__ inline int dg_neighbours(const GridDesc& g, long long e, bool with_self, long long* nb) {
  int cnt = 0;
  if (!g.simplex) {
    long long ci[3];
    cell_multi(g, e, ci);
    // -z, -y, -x, self, +x, +y, +z is ascending in the lexicographic index
    for (int k = g.dim - 1; k >= 0; --k)
      if (ci[k] > 0) {
        long long cj[3] = {ci[0], ci[1], ci[2]};
        cj[k] -= 1;
        nb[cnt++] = cell_index(g, cj);
      }
    if (with_self) nb[cnt++] = e;
    for (int k = 0; k < g.dim; ++k)
      if (ci[k] < g.n[k] - 1) {
        long long cj[3] = {ci[0], ci[1], ci[2]};
        cj[k] += 1;
        nb[cnt++] = cell_index(g, cj);
      }
    return cnt;
  }
  // 2D Kuhn: e = 2c + t
  long long c = e >> 1;
  int t = int(e & 1);
  long long ci[3];
  cell_multi(g, c, ci);
  if (t == 0) {  // A: faces bottom (to B below), diagonal (B same cube), right (B right)
    if (ci[1] > 0) nb[cnt++] = 2 * (c - g.n[0]) + 1;
    if (with_self) nb[cnt++] = e;
    nb[cnt++] = 2 * c + 1;
    if (ci[0] < g.n[0] - 1) nb[cnt++] = 2 * (c + 1) + 1;
  } else {  // B: faces left (A left), diagonal (A same cube), top (A above)
    if (ci[0] > 0) nb[cnt++] = 2 * (c - 1);
    nb[cnt++] = 2 * c;
    if (with_self) nb[cnt++] = e;
    if (ci[1] < g.n[1] - 1) nb[cnt++] = 2 * (c + g.n[0]);
  }
  return cnt;
}

}  // namespace gdt
