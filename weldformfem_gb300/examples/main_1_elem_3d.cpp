// One-hexahedron compression driven through the C++ facade, written the way
// the reference's example driver is (src/common/main_1_elem_3d.C): AddBoxLength,
// setDensity, AssignMaterial, AddBCVelNode, AllocateBCs, SetDT, SetEndTime,
// SolveChungHulbert. Prints the node displacements, one node per line.
//
// Build: g++ -std=c++17 -I include weldformfem_gb300/examples/main_1_elem_3d.cpp \
//        -L weldformfem_gb300/_lib -lwf_gb300 -Wl,-rpath,weldformfem_gb300/_lib
#include <cstdio>
#include <cstdlib>

#include "weldform/Domain.h"

using namespace weldform;

int main(int argc, char **argv) {
  const int precision = (argc > 1) ? std::atoi(argv[1]) : WF_FP64;
  try {
    Domain_d dom(precision);
    const double3 V = make_double3(0.0, 0.0, 0.0);
    const double dx = 0.1;
    const double3 L = make_double3(dx, dx, dx);
    const double r = 0.05;
    dom.AddBoxLength(V, L, r, true);
    const double E = 206.0e9, nu = 0.3, rho = 7850.0;
    dom.setDensity(rho);
    Elastic_ el(E, nu);
    Material_ mat(el);
    mat.Material_model = BILINEAR;
    dom.AssignMaterial(&mat);
    const double dt = 0.800e-5;
    dom.SetDT(dt);
    dom.SetEndTime(1.0e-3);
    dom.AddBCVelNode(0, 0, 0); dom.AddBCVelNode(0, 1, 0); dom.AddBCVelNode(0, 2, 0);
    dom.AddBCVelNode(1, 1, 0); dom.AddBCVelNode(1, 2, 0);
    dom.AddBCVelNode(2, 0, 0); dom.AddBCVelNode(2, 2, 0);
    dom.AddBCVelNode(3, 2, 0);
    for (int i = 0; i < 4; i++) dom.AddBCVelNode(i + 4, 2, -1.0);
    dom.AllocateBCs();
    dom.SolveChungHulbert();
    for (int n = 0; n < dom.getNodeCount(); n++) {
      const double3 u = dom.getDispVec(n);
      std::printf("%.17e %.17e %.17e\n", u.x, u.y, u.z);
    }
  } catch (const std::exception &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
