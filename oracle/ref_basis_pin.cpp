// ref_basis_pin.cpp — compiles the reference's own basis function tables
// where they lie (include/FE3D/BF_C_H_Q2_3D.h and BF_D_H_P1_3D.h for the
// hexahedron; BF_C_T_B2_3D.h, P2 with 4 face and 1 cell bubbles, and
// BF_D_T_P1_3D.h for the tetrahedron; they contain only arithmetic) against a
// minimal stand-in for the TBaseFunct3D constructor they call, and prints
// their values and first derivatives at fixed points as JSON (argument "tet"
// selects the tetrahedral pair).  The outputs are the golden fixtures
// tests/golden/basis_q2_p1.json and basis_tet_b2_p1.json (generator:
// tests/golden/make_basis_golden.py).  TEST INFRASTRUCTURE ONLY.
#include <cstdio>

typedef void DoubleFunct3D(double, double, double, double *);
#include <cstring>
enum BaseFunct3D { BF_C_H_Q2_3D, BF_D_H_P1_3D, BF_C_T_B2_3D, BF_D_T_P1_3D };
enum BF3DRefElements { BFUnitTetrahedron, BFUnitHexahedron };
class TBaseFunct3D {
 public:
  TBaseFunct3D(int, BaseFunct3D, BF3DRefElements, DoubleFunct3D *, DoubleFunct3D *,
               DoubleFunct3D *, DoubleFunct3D *, DoubleFunct3D *, DoubleFunct3D *,
               DoubleFunct3D *, DoubleFunct3D *, DoubleFunct3D *, DoubleFunct3D *, int, int, int,
               int ***, int = 1) {}
};

#include <BF_C_H_Q2_3D.h>
#include <BF_D_H_P1_3D.h>
#include <BF_C_T_B2_3D.h>
#include <BF_D_T_P1_3D.h>

static void emit(const char *name, int n, DoubleFunct3D *f, double x, double y, double z,
                 bool last) {
  double v[32];
  f(x, y, z, v);
  std::printf("\"%s\": [", name);
  for (int i = 0; i < n; ++i) std::printf("%.17g%s", v[i], i + 1 < n ? ", " : "");
  std::printf("]%s", last ? "" : ", ");
}

static int tet_main() {
  // points of the reference tetrahedron (0,0,0), (1,0,0), (0,1,0), (0,0,1):
  // vertices, edge midpoints, face and cell barycentres, interior points
  const double pts[][3] = {{0, 0, 0},       {1, 0, 0},       {0, 1, 0},       {0, 0, 1},
                           {0.5, 0.5, 0},   {0, 0.5, 0.5},   {1.0 / 3, 1.0 / 3, 1.0 / 3},
                           {0.25, 0.25, 0.25}, {0.1, 0.2, 0.3}, {0.6, 0.1, 0.05},
                           {0.05, 0.7, 0.2}, {0.3, 0.3, 0.1}, {0.15, 0.05, 0.65},
                           {0.2, 0.45, 0.2}};
  const int np = sizeof(pts) / sizeof(pts[0]);
  std::printf("{\"points\": [");
  for (int p = 0; p < np; ++p)
    std::printf("[%.17g, %.17g, %.17g]%s", pts[p][0], pts[p][1], pts[p][2], p + 1 < np ? ", " : "");
  std::printf("], \"values\": [");
  for (int p = 0; p < np; ++p) {
    const double x = pts[p][0], y = pts[p][1], z = pts[p][2];
    std::printf("{");
    emit("b2", 15, C_T_B2_3D_Funct, x, y, z, false);
    emit("b2_xi", 15, C_T_B2_3D_DeriveXi, x, y, z, false);
    emit("b2_eta", 15, C_T_B2_3D_DeriveEta, x, y, z, false);
    emit("b2_zeta", 15, C_T_B2_3D_DeriveZeta, x, y, z, false);
    emit("p1", 4, D_T_P1_3D_Funct, x, y, z, false);
    emit("p1_xi", 4, D_T_P1_3D_DeriveXi, x, y, z, false);
    emit("p1_eta", 4, D_T_P1_3D_DeriveEta, x, y, z, false);
    emit("p1_zeta", 4, D_T_P1_3D_DeriveZeta, x, y, z, true);
    std::printf("}%s", p + 1 < np ? ", " : "");
  }
  std::printf("]}\n");
  return 0;
}

int main(int argc, char **argv) {
  if (argc > 1 && std::strcmp(argv[1], "tet") == 0) return tet_main();
  const double pts[][3] = {{-1, -1, -1}, {0, 0, 0},        {1, 1, 1},        {1, -1, 0},
                           {-1, 0, 1},   {0.5, 0.5, -0.5}, {-0.5, 0.25, 0.75}, {0.3, -0.7, 0.1},
                           {-0.9, 0.6, -0.2}, {0.125, -0.375, 0.625}, {0.861, -0.34, 0.34},
                           {-0.57735, 0.57735, -0.57735}};
  const int np = sizeof(pts) / sizeof(pts[0]);
  std::printf("{\"points\": [");
  for (int p = 0; p < np; ++p)
    std::printf("[%.17g, %.17g, %.17g]%s", pts[p][0], pts[p][1], pts[p][2], p + 1 < np ? ", " : "");
  std::printf("], \"values\": [");
  for (int p = 0; p < np; ++p) {
    const double x = pts[p][0], y = pts[p][1], z = pts[p][2];
    std::printf("{");
    emit("q2", 27, C_H_Q2_3D_Funct, x, y, z, false);
    emit("q2_xi", 27, C_H_Q2_3D_DeriveXi, x, y, z, false);
    emit("q2_eta", 27, C_H_Q2_3D_DeriveEta, x, y, z, false);
    emit("q2_zeta", 27, C_H_Q2_3D_DeriveZeta, x, y, z, false);
    emit("p1", 4, D_H_P1_3D_Funct, x, y, z, false);
    emit("p1_xi", 4, D_H_P1_3D_DeriveXi, x, y, z, false);
    emit("p1_eta", 4, D_H_P1_3D_DeriveEta, x, y, z, false);
    emit("p1_zeta", 4, D_H_P1_3D_DeriveZeta, x, y, z, true);
    std::printf("}%s", p + 1 < np ? ", " : "");
  }
  std::printf("]}\n");
  return 0;
}
