// Entries of the augmented Kansa matrix K = [[op(Phi), op(P)], [bd(Phi), bd(P)], [P^T, 0]] by row and column
// (FP64, closed-form kernel derivatives), shared by the tiled assembly and the batched solver.
//
// Rows r < Ni apply the captured operator (updes/assembly.py:93-137), Ni <= r < N the boundary conditions
// (assembly.py:141-362), r >= N are the P^T rows of assemble_A (assembly.py:62-85).
#pragma once

#include "common.cuh"
#include "rbf.cuh"

struct RowInfo {
  int kind;  // -1 interior, -2 P^T row, else UPDES_ROW_*
  int a, b;  // evaluation node, partner node
  double xa, ya, xb, yb;
  double w0, w1, w2, w3, w4;  // interior: value, d/dx, d/dy, d2/dx2, d2/dy2
  double n1x, n1y, n2x, n2y, nPx, nPy, beta;
};

__device__ __forceinline__ RowInfo load_row(const updes_problem& p, int r) {
  RowInfo ri;
  if (r < p.Ni) {
    ri.kind = -1;
    ri.a = ri.b = r;
    const double* w = p.op_weights + 5ll * r;
    ri.w0 = w[0]; ri.w1 = w[1]; ri.w2 = w[2]; ri.w3 = w[3]; ri.w4 = w[4];
    ri.n1x = ri.n1y = ri.n2x = ri.n2y = ri.nPx = ri.nPy = ri.beta = 0.0;
  } else if (r < p.N) {
    const int b = r - p.Ni;
    ri.kind = p.bd_kind[b];
    ri.a = p.bd_node[2 * b];
    ri.b = p.bd_node[2 * b + 1];
    const double* g = p.bd_geom + 8ll * b;
    ri.n1x = g[0]; ri.n1y = g[1]; ri.n2x = g[2]; ri.n2y = g[3];
    ri.nPx = g[4]; ri.nPy = g[5]; ri.beta = g[6];
    ri.w0 = ri.w1 = ri.w2 = ri.w3 = ri.w4 = 0.0;
  } else {
    ri.kind = -2;
    ri.a = ri.b = r - p.N;  // monomial id
    ri.w0 = ri.w1 = ri.w2 = ri.w3 = ri.w4 = 0.0;
    ri.n1x = ri.n1y = ri.n2x = ri.n2y = ri.nPx = ri.nPy = ri.beta = 0.0;
    ri.xa = ri.ya = ri.xb = ri.yb = 0.0;
    return ri;
  }
  ri.xa = p.nodes[2ll * ri.a];
  ri.ya = p.nodes[2ll * ri.a + 1];
  ri.xb = p.nodes[2ll * ri.b];
  ri.yb = p.nodes[2ll * ri.b + 1];
  return ri;
}

// Entry (row, node column c) of K for c < N.
template <int KIND>
__device__ __forceinline__ double entry_rbf(const RowInfo& ri, int c, double xc, double yc, double param,
                                            int ip, int self_term) {
  if (ri.kind == -2) {  // P^T row: monomial(ri.a) at node c
    const MonoT m = monomial_terms(ri.a, xc, yc);
    return m.m;
  }
  const double dx = ri.xa - xc, dy = ri.ya - yc;
  const double r2 = dx * dx + dy * dy;
  if (ri.kind == -1) {
    if (c == ri.a && !self_term) return 0.0;
    if (r2 == 0.0) return ri.w0 * rbf_phi0<KIND>();
    const RbfG g = rbf_g<KIND>(r2, param, ip);
    return ri.w0 * g.phi + g.g1 * (ri.w1 * dx + ri.w2 * dy + (ri.w3 + ri.w4)) +
           g.g2 * (ri.w3 * dx * dx + ri.w4 * dy * dy);
  }
  if (ri.kind <= UPDES_ROW_ROBIN) {
    if (c == ri.a && !self_term) return 0.0;
    if (r2 == 0.0) return (ri.kind == UPDES_ROW_NEUMANN) ? 0.0 : (ri.kind == UPDES_ROW_ROBIN ? ri.beta : 1.0) * rbf_phi0<KIND>();
    const RbfG g = rbf_g<KIND>(r2, param, ip);
    if (ri.kind == UPDES_ROW_DIRICHLET) return g.phi;
    const double fl = g.g1 * (ri.n1x * dx + ri.n1y * dy);
    if (ri.kind == UPDES_ROW_NEUMANN) return fl;
    return ri.beta * g.phi + fl;
  }
  // periodic rows span every column
  const double ex = ri.xb - xc, ey = ri.yb - yc;
  const double s2 = ex * ex + ey * ey;
  RbfG ga, gb;
  if (r2 == 0.0) { ga.phi = rbf_phi0<KIND>(); ga.g1 = 0.0; ga.g2 = 0.0; } else ga = rbf_g<KIND>(r2, param, ip);
  if (s2 == 0.0) { gb.phi = rbf_phi0<KIND>(); gb.g1 = 0.0; gb.g2 = 0.0; } else gb = rbf_g<KIND>(s2, param, ip);
  if (ri.kind == UPDES_ROW_PERIODIC_VALUE) return ga.phi - gb.phi;
  return ga.g1 * (ri.n1x * dx + ri.n1y * dy) + gb.g1 * (ri.n2x * ex + ri.n2y * ey);
}

// entry_rbf for a row whose evaluation node is also its value row's node (every row r < N but the periodic
// flux rows), returning as well the value-row entry A[a][c] = phi(x_a - x_c) (0 at c = a unless self_term)
// from the same kernel evaluation.
template <int KIND>
__device__ __forceinline__ double entry_rbf_phi(const RowInfo& ri, int c, double xc, double yc, double param,
                                                int ip, int self_term, double* phi) {
  const double dx = ri.xa - xc, dy = ri.ya - yc;
  const double r2 = dx * dx + dy * dy;
  if (c == ri.a && !self_term) {
    *phi = 0.0;
    if (ri.kind == UPDES_ROW_PERIODIC_VALUE || ri.kind == UPDES_ROW_PERIODIC_FLUX)
      return entry_rbf<KIND>(ri, c, xc, yc, param, ip, self_term);
    return 0.0;
  }
  if (ri.kind == UPDES_ROW_PERIODIC_VALUE || ri.kind == UPDES_ROW_PERIODIC_FLUX || r2 == 0.0) {
    *phi = r2 == 0.0 ? rbf_phi0<KIND>() : rbf_g<KIND>(r2, param, ip).phi;
    return entry_rbf<KIND>(ri, c, xc, yc, param, ip, self_term);
  }
  const RbfG g = rbf_g<KIND>(r2, param, ip);
  *phi = g.phi;
  if (ri.kind == -1)
    return ri.w0 * g.phi + g.g1 * (ri.w1 * dx + ri.w2 * dy + (ri.w3 + ri.w4)) +
           g.g2 * (ri.w3 * dx * dx + ri.w4 * dy * dy);
  if (ri.kind == UPDES_ROW_DIRICHLET) return g.phi;
  const double fl = g.g1 * (ri.n1x * dx + ri.n1y * dy);
  if (ri.kind == UPDES_ROW_NEUMANN) return fl;
  return ri.beta * g.phi + fl;
}

// Entry (row, monomial column k) of K.
__device__ __forceinline__ double entry_mono(const RowInfo& ri, int k) {
  if (ri.kind == -2) return 0.0;
  const MonoT m = monomial_terms(k, ri.xa, ri.ya);
  switch (ri.kind) {
    case -1:
      return ri.w0 * m.m + ri.w1 * m.mx + ri.w2 * m.my + ri.w3 * m.mxx + ri.w4 * m.myy;
    case UPDES_ROW_DIRICHLET:
      return m.m;
    case UPDES_ROW_NEUMANN:
      return m.mx * ri.nPx + m.my * ri.nPy;
    case UPDES_ROW_ROBIN:
      return ri.beta * m.m + (m.mx * ri.nPx + m.my * ri.nPy);
    case UPDES_ROW_PERIODIC_VALUE: {
      const MonoT q = monomial_terms(k, ri.xb, ri.yb);
      return m.m - q.m;
    }
    default: {
      const MonoT q = monomial_terms(k, ri.xb, ri.yb);
      return (m.mx * ri.n1x + m.my * ri.n1y) + (q.mx * ri.n2x + q.my * ri.n2y);
    }
  }
}
