// One event through the MCnucl call surface (MCnucl.h), as the reference's
// operations drive MCnucl: generateNuclei(b) until the event has a binary
// collision and passes the centrality cut, then the thickness and density,
// then the order-2 reaction-plane and participant-plane frames.  Reads
// parameters.dat and key=value arguments (b=<impact parameter>); writes into
// the working directory: mcnucl_meta.txt (b, Npart1, Npart2, Ncoll, dN/dy of
// each frame, the orientations), mcnucl_nuclei.txt (x y per nucleon,
// projectile then target) and the FP32 grids ta.f32, tb.f32, rho.f32,
// rho_rp2.f32, rho_pp2.f32 ([nx][ny] each).
#include <cstdio>
#include <string>
#include <vector>

#include "MCnucl.h"
#include "ParameterReader.h"

namespace {

void write_grid(const smc::MCnucl &mc, const char *name, int which) {
  const int nx = mc.info().nx, ny = mc.info().ny;
  std::vector<float> g((size_t)nx * ny);
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      g[(size_t)i * ny + j] = (float)(which == 0 ? mc.getTA1(i, j) : which == 1 ? mc.getTA2(i, j) : mc.getRho(0, i, j));
  FILE *f = std::fopen(name, "wb");
  std::fwrite(g.data(), sizeof(float), g.size(), f);
  std::fclose(f);
}

}  // namespace

int main(int argc, char *argv[]) {
  try {
    smc::ParameterReader reader;
    reader.readFromFile("parameters.dat");
    reader.readFromArguments(argc, argv);
    const double b = reader.getVal("b", 6.0);
    smc::MCnucl mc(&reader);
    int tries = 0;
    do {
      if (tries++) mc.deleteNucleus();
      mc.generateNuclei(b);
    } while ((mc.getBinaryCollision() == 0 || mc.CentralityCut() == 0) && tries < 1000);
    mc.calculateThickness();
    mc.setDensity(0, -1);
    const double dndy = mc.getdNdy();
    write_grid(mc, "ta.f32", 0);
    write_grid(mc, "tb.f32", 1);
    write_grid(mc, "rho.f32", 2);
    mc.recenterGrid(0, 2);
    mc.calculateThickness();
    mc.setDensity(0, -1);
    const double dndy_rp = mc.getdNdy();
    write_grid(mc, "rho_rp2.f32", 2);
    mc.rotateGrid(0, 2);
    mc.calculateThickness();
    mc.setDensity(0, -1);
    const double dndy_pp = mc.getdNdy();
    write_grid(mc, "rho_pp2.f32", 2);
    FILE *f = std::fopen("mcnucl_meta.txt", "w");
    std::fprintf(f, "%.17g %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %d\n", mc.impactParameter(),
                 mc.getNpart1(), mc.getNpart2(), mc.getNcoll(), dndy, dndy_rp, dndy_pp, mc.lastCx1, mc.lastPh1,
                 mc.lastCx2, mc.lastPh2, tries);
    std::fclose(f);
    f = std::fopen("mcnucl_nuclei.txt", "w");
    for (size_t k = 0; k + 1 < mc.projectile().size(); k += 2)
      std::fprintf(f, "%.17g %.17g\n", mc.projectile()[k], mc.projectile()[k + 1]);
    for (size_t k = 0; k + 1 < mc.target().size(); k += 2)
      std::fprintf(f, "%.17g %.17g\n", mc.target()[k], mc.target()[k + 1]);
    std::fclose(f);
    mc.dumpBinaryTable("data/binary.dat");
  } catch (const std::exception &e) {
    std::fprintf(stderr, "mcnucl_event: %s\n", e.what());
    return 1;
  }
  return 0;
}
