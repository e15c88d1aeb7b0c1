// Hex-element geometry shared by the host set-up code and the device kernels.
//
// Corner area normals (the "B matrix", Explicit-Lagrange-Kokkos/SGH_solver/
// geometry.cpp:40-234) and the exact trilinear volume (geometry.cpp:271-310) are
// cofactor sums whose term order fixes their rounding, so they are encoded here as
// tables in exactly that order (the tables are data, the evaluation code is ours):
//
//   B(p,c) = ( sum_{t=0..5} O[J[p][t]] * comb(p,t)(I) ) / 12,  left to right,
//   (O, I) = (y, z), (z, x), (x, y) for c = 0, 1, 2,
//   comb(p,t)(I) = signed I-values summed left to right, TERMS[p][t] encoded as
//   +-(node+1), 0 = unused;
//   V = ( sum_a x[VI[a]] * (sum_b y[VJ[a][b]] * comb(VI[a], VJ[a][b])(z)) ) / 12.
//
// Two exact identities make work shareable without changing a single bit:
// comb(j,p) is the term-by-term negation of comb(p,j) (floating-point negation is
// exact and rounding is sign-symmetric), and the volume's inner combos are the
// B-matrix combos of the same (i, j) pair.
#ifndef FIERRO_SGH_HEX_H
#define FIERRO_SGH_HEX_H

#ifdef __CUDACC__
#define FIERRO_HD __host__ __device__ __forceinline__
#else
#define FIERRO_HD inline
#endif

namespace fierro {
namespace hex {

// Neighbour node of corner p for each of the six product terms, summation order.
constexpr int J[8][6] = {
    {1, 2, 3, 4, 5, 7}, {0, 2, 3, 4, 5, 6}, {0, 1, 3, 5, 6, 7}, {0, 1, 2, 4, 6, 7},
    {0, 1, 3, 5, 6, 7}, {0, 1, 2, 4, 6, 7}, {1, 2, 3, 4, 5, 7}, {0, 2, 3, 4, 5, 6},
};
constexpr signed char TERMS[8][6][4] = {
    {{-3, -4, 5, 6}, {2, -4, 0, 0}, {2, 3, -5, -8}, {-2, 4, -6, 8}, {-2, 5, 0, 0}, {4, -5, 0, 0}},
    {{3, 4, -5, -6}, {-1, -4, 6, 7}, {-1, 3, 0, 0}, {1, -6, 0, 0}, {1, -3, 5, -7}, {-3, 6, 0, 0}},
    {{-2, 4, 0, 0}, {1, 4, -6, -7}, {-1, -2, 7, 8}, {2, -7, 0, 0}, {2, -4, 6, -8}, {-4, 7, 0, 0}},
    {{-2, -3, 5, 8}, {1, -3, 0, 0}, {1, 2, -7, -8}, {-1, 8, 0, 0}, {3, -8, 0, 0}, {-1, 3, -5, 7}},
    {{2, -4, 6, -8}, {-1, 6, 0, 0}, {1, -8, 0, 0}, {-1, -2, 7, 8}, {-6, 8, 0, 0}, {1, 4, -6, -7}},
    {{2, -5, 0, 0}, {-1, 3, -5, 7}, {-2, 7, 0, 0}, {1, 2, -7, -8}, {-2, -3, 5, 8}, {5, -7, 0, 0}},
    {{3, -6, 0, 0}, {-2, 4, -6, 8}, {-3, 8, 0, 0}, {6, -8, 0, 0}, {2, 3, -5, -8}, {-3, -4, 5, 6}},
    {{-4, 5, 0, 0}, {4, -7, 0, 0}, {1, -3, 5, -7}, {-1, -4, 6, 7}, {-5, 7, 0, 0}, {3, 4, -5, -6}},
};
constexpr int VI[8] = {1, 7, 3, 5, 6, 0, 2, 4};
constexpr int VJ[8][6] = {
    {3, 4, 0, 6, 5, 2}, {0, 6, 2, 3, 5, 4}, {1, 7, 6, 2, 4, 0}, {0, 7, 2, 1, 4, 6},
    {1, 7, 5, 4, 3, 2}, {2, 7, 5, 1, 3, 4}, {0, 5, 1, 7, 6, 3}, {1, 7, 3, 0, 6, 5},
};
// Face (patch) node lids, mesh.h:352-357.
constexpr int PATCH[6][4] = {
    {0, 4, 7, 3}, {1, 2, 6, 5}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 3, 2, 1}, {4, 5, 6, 7},
};
// Position t of neighbour j in row p of J (compile-time).
constexpr int slot(int p, int j) {
  return J[p][0] == j ? 0 : J[p][1] == j ? 1 : J[p][2] == j ? 2 : J[p][3] == j ? 3 : J[p][4] == j ? 4 : 5;
}

// Signed sum of I over one TERMS row, left to right.
FIERRO_HD double comb(const signed char* t, const double* I) {
  double s = (t[0] > 0) ? I[t[0] - 1] : -I[-t[0] - 1];
  for (int k = 1; k < 4; ++k) {
    if (t[k] > 0) s = s + I[t[k] - 1];
    else if (t[k] < 0) s = s - I[-t[k] - 1];
  }
  return s;
}

// Outward corner area normals B[p][c] of one hex (geometry.cpp:40-234).
FIERRO_HD void bmatrix(const double* x, const double* y, const double* z, double B[8][3]) {
  const double twelth = 1. / 12.;
  const double* O[3] = {y, z, x};
  const double* I[3] = {z, x, y};
  for (int c = 0; c < 3; ++c)
    for (int p = 0; p < 8; ++p) {
      double acc = O[c][J[p][0]] * comb(TERMS[p][0], I[c]);
      for (int t = 1; t < 6; ++t) acc = acc + O[c][J[p][t]] * comb(TERMS[p][t], I[c]);
      B[p][c] = acc * twelth;
    }
}

// Exact hex volume (geometry.cpp:271-310).
FIERRO_HD double volume(const double* x, const double* y, const double* z) {
  const double twelth = 1. / 12.;
  double vol = 0.0;
  for (int a = 0; a < 8; ++a) {
    const int i = VI[a];
    double inner = y[VJ[a][0]] * comb(TERMS[i][slot(i, VJ[a][0])], z);
    for (int b = 1; b < 6; ++b) inner = inner + y[VJ[a][b]] * comb(TERMS[i][slot(i, VJ[a][b])], z);
    vol = (a == 0) ? x[i] * inner : vol + x[i] * inner;
  }
  return vol * twelth;
}

}  // namespace hex
}  // namespace fierro

#endif
