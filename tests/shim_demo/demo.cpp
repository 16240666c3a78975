// A caller of the reference's solver class, built against include/magnetic_force.cuh
// and libmfgb.so.  It follows the call sequence of the reference's demo
// (magnetic_solver/main.cu:3-62): a 2x2x2 unit lattice, one external dipole,
// solve, force, move the targets, new external field, solve, force, export.
//   usage: demo <out_dir>
#include <cstdio>
#include <string>
#include <vector>

#include "magnetic_force.cuh"

int main(int argc, char** argv) {
  const std::string out = argc > 1 ? argv[1] : ".";
  std::vector<float3> lattice, moved;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j)
      for (int k = 0; k < 2; ++k) {
        lattice.push_back(make_float3(float(i), float(j), float(k)));
        if (k == 0) moved.push_back(make_float3(float(i), float(j), 1.f));
      }
  std::vector<float3> src_pos{make_float3(0.f, 0.f, 0.f)};
  std::vector<float3> src_m{make_float3(0.f, 1.f, 0.f)};
  float H0[3] = {0.f, 1.f, 0.f};
  Libo::cuda_magnet_cgOptimizer::CtorParam p{lattice.size(), 1.f, 1.f, 1.f, 1.f, H0, src_pos, src_m, lattice};
  Libo::cuda_magnet_cgOptimizer solver{p};
  solver.solve(100);
  solver.evaluate_fitted_near_foece();
  std::printf("first solve: %zu steps, %zu errors recorded, last %.6e\n", solver.i_step,
              solver.total_error.size(), solver.total_error.empty() ? 0.0 : solver.total_error.back());
  solver.export_data((out + "/first_data.txt").c_str());
  solver.export_force((out + "/first_force.txt").c_str());

  solver.setTargetpos(moved);
  Libo::cuda_magnet_cgOptimizer::setHextParams hp;
  hp.const_ext_field[0] = H0[0];
  hp.const_ext_field[1] = H0[1];
  hp.const_ext_field[2] = H0[2];
  hp.ext_source_pos = src_pos;
  hp.ext_source_M = src_m;
  hp.ext_mag_h = 1.f;
  solver.setHext(hp);
  solver.solve(100);
  solver.evaluate_fitted_near_foece();
  // read a published member directly, as a caller of the reference would
  std::vector<float> fx, fy, fz;
  solver.magnetic_bodyforce.export_data(fx, fy, fz);
  std::printf("second solve: np=%zu F0=(%.6e, %.6e, %.6e)\n", solver.np, fx[0], fy[0], fz[0]);
  solver.export_data((out + "/temp.txt").c_str());
  solver.export_force((out + "/force.txt").c_str());
  return 0;
}
