// host_classes.cpp -- drives the C++ host classes of include/mlgpu.hpp on one
// GPU with the reference's method names: reads the fields written by
// tests/test_cpp_host.py, runs residual / levelGSRB / MGnewOp + restrictR +
// applyOp / an AMRFASMultiGrid solve and TGA step / an AMRMultiGrid projection
// solve, and writes each result for comparison with the oracle.
// Usage: host_classes <dir> <nx> <ny>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "mlgpu.hpp"

static std::vector<double> load(const std::string &path, size_t n) {
  std::vector<double> v(n);
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(double), n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

static void save(const std::string &path, const std::vector<double> &v) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f || std::fwrite(v.data(), sizeof(double), v.size(), f) != v.size()) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
}

static std::vector<double> fetch(const mlgpu::DeviceField &f) {
  std::vector<double> v(f.size());
  f.download(v.data());
  return v;
}

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  const std::string dir = argv[1];
  const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]);
  const mlgpu_grid g = {2, {nx, ny, 1}, 1.0 / nx, {0, 0, 0}};
  const size_t nc = (size_t)nx * ny;
  try {
    // ---- nonlinear (H, C) operator: the diffusive solidification setting
    mlgpu::DeviceField bx(g, 2, MLGPU_F64, mlgpu::faces(g, 0));
    mlgpu::DeviceField by(g, 2, MLGPU_F64, mlgpu::faces(g, 1));
    bx.upload(load(dir + "/bx.bin", 2 * mlgpu::faces(g, 0)).data());
    by.upload(load(dir + "/by.bin", 2 * mlgpu::faces(g, 1)).data());
    mlgpu_nlop d = {};
    d.grid = g;
    d.params.compositionRatio = 5.0;
    d.params.waterDistributionCoeff = 1e-3;
    d.params.specificHeatRatio = 1.0;
    d.params.stefan = 5.0;
    d.derived_bc.type[1][0][0] = d.derived_bc.type[1][0][1] = MLGPU_BC_DIRICHLET;
    d.derived_bc.type[1][1][0] = d.derived_bc.type[1][1][1] = MLGPU_BC_DIRICHLET;
    d.derived_bc.value[1][0][0] = -1.0;
    d.derived_bc.value[1][0][1] = -1.0;
    d.derived_bc.value[1][1][0] = 0.5;
    d.derived_bc.value[1][1][1] = -1.0;
    d.apply_derived_bc = 1;
    d.alpha = 1.0;
    d.beta = -1e-3;
    d.bCoef[0] = bx.data();
    d.bCoef[1] = by.data();
    d.dtype = MLGPU_F64;
    mlgpu::NLMultiCompOp op(d);

    mlgpu::DeviceField phi(g, 2), rhs(g, 2), res(g, 2);
    const std::vector<double> phi_h = load(dir + "/phi.bin", 2 * nc);
    phi.upload(phi_h.data());
    rhs.upload(load(dir + "/rhs.bin", 2 * nc).data());
    op.residual(res, phi, rhs);
    save(dir + "/out_residual.bin", fetch(res));

    mlgpu::DeviceField sm(g, 2);
    sm.copyFrom(phi);
    op.levelGSRB(sm, rhs);
    save(dir + "/out_gsrb.bin", fetch(sm));

    std::unique_ptr<mlgpu::NLMultiCompOp> coarse = op.MGnewOp();
    std::unique_ptr<mlgpu::DeviceField> pc = op.createCoarser(phi);
    op.restrictR(*pc, phi);
    mlgpu::DeviceField lc(pc->grid(), 2);
    coarse->applyOp(lc, *pc);
    save(dir + "/out_coarse_apply.bin", fetch(lc));

    mlgpu::DeviceField u(g, 2);
    u.copyFrom(phi);
    mlgpu::AMRFASMultiGrid fas(op);
    const mlgpu_solve_stats st = fas.solve(u, rhs);
    save(dir + "/out_fas.bin", fetch(u));
    // one TGA step from phi (dt 1e-3) on the same solver
    mlgpu::DeviceField ut(g, 2);
    ut.copyFrom(phi);
    fas.tgaStep(ut, phi, 1e-3);
    save(dir + "/out_tga.bin", fetch(ut));

    // ---- projection operator: div(Pi grad p) = f, Neumann walls
    mlgpu::DeviceField p0(g, 1, MLGPU_F64, mlgpu::faces(g, 0));
    mlgpu::DeviceField p1(g, 1, MLGPU_F64, mlgpu::faces(g, 1));
    p0.upload(load(dir + "/pb0.bin", mlgpu::faces(g, 0)).data());
    p1.upload(load(dir + "/pb1.bin", mlgpu::faces(g, 1)).data());
    mlgpu_vcop v = {};
    v.grid = g;
    v.alpha = 0.0;
    v.beta = 1.0;
    v.bCoef[0] = p0.data();
    v.bCoef[1] = p1.data();
    v.dtype = MLGPU_F64;
    mlgpu::ProjectionOp pop(v);
    mlgpu::DeviceField f(g, 1), p(g, 1);
    f.upload(load(dir + "/f.bin", nc).data());
    // the projection operator one level coarser applied to the averaged f
    std::unique_ptr<mlgpu::VCOp> pc_op = pop.MGnewOp();
    std::unique_ptr<mlgpu::DeviceField> fc = pop.createCoarser(f);
    pop.restrictR(*fc, f);
    mlgpu::DeviceField lfc(fc->grid(), 1);
    pc_op->applyOp(lfc, *fc);
    save(dir + "/out_projection_coarse_apply.bin", fetch(lfc));
    p.setToZero();
    mlgpu::AMRMultiGrid mg(pop);
    const mlgpu_solve_stats sp = mg.solve(p, f);
    save(dir + "/out_projection.bin", fetch(p));

    std::printf("{\"fas_iterations\": %d, \"fas_status\": %d, \"projection_iterations\": %d, "
                "\"projection_status\": %d}\n",
                st.iterations, st.exit_status, sp.iterations, sp.exit_status);
  } catch (const mlgpu::Error &e) {
    std::fprintf(stderr, "mlgpu error: %s\n", e.what());
    return 1;
  }
  return 0;
}
