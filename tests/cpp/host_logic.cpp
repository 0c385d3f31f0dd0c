// host_logic.cpp -- the host-side logic of include/mlgpu.hpp that needs no
// GPU: box arithmetic, the coarsening limit of the factories, and the
// mapping of status codes to mlgpu::Error.  Prints "ok" and exits 0 when all
// checks hold.
#include <cstdio>
#include <string>

#include "mlgpu.hpp"

#define EXPECT(c)                                          \
  do {                                                     \
    if (!(c)) {                                            \
      std::fprintf(stderr, "check failed: %s\n", #c);      \
      return 1;                                            \
    }                                                      \
  } while (0)

int main() {
  const mlgpu_grid g = {2, {8, 6, 1}, 0.125, {1, 0, 0}};
  EXPECT(mlgpu::cells(g) == 48);
  EXPECT(mlgpu::faces(g, 0) == 9 * 6);
  EXPECT(mlgpu::faces(g, 1) == 8 * 7);
  EXPECT(mlgpu::coarsenable(g));
  const mlgpu_grid c = mlgpu::coarsened(g);
  EXPECT(c.n[0] == 4 && c.n[1] == 3 && c.n[2] == 1 && c.dx == 0.25 && c.periodic[0] == 1);
  EXPECT(!mlgpu::coarsenable(c));  // 3 cells along y: the coarsening limit
  const mlgpu_grid g3 = {3, {4, 4, 2}, 0.25, {0, 0, 0}};
  EXPECT(mlgpu::cells(g3) == 32 && mlgpu::faces(g3, 2) == 48);

  // status codes become exceptions carrying the status and its text
  try {
    mlgpu::check(MLGPU_ERR_ARG, "call");
    return 1;
  } catch (const mlgpu::Error &e) {
    EXPECT(e.status() == MLGPU_ERR_ARG);
    EXPECT(std::string(e.what()).find("invalid argument") != std::string::npos);
  }
  // MGnewOp at the coarsening limit is nullptr, without touching the device
  mlgpu_nlop d = {};
  d.grid = c;
  d.dtype = MLGPU_F64;
  mlgpu::NLMultiCompOp op(d);
  EXPECT(op.MGnewOp() == nullptr);
  mlgpu_vcop v = {};
  v.grid = c;
  v.dtype = MLGPU_F64;
  mlgpu::ProjectionOp pop(v);
  EXPECT(pop.MGnewOp() == nullptr);
  // invalid descriptors are refused before any device work
  mlgpu_mg_options o = mlgpu::default_options(true);
  o.relax_mode = 7;
  try {
    mlgpu::AMRFASMultiGrid fas(op, o);
    return 1;
  } catch (const mlgpu::Error &e) {
    EXPECT(e.status() == MLGPU_ERR_ARG);
  }
  std::printf("ok\n");
  return 0;
}
