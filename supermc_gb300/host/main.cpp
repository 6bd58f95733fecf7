// Drop-in for the reference's driver (src/main.cpp:19-73): parameters.dat then
// key=value arguments, then the operation's event loop on the GPU.
#include <cstdio>
#include <ctime>

#include "MakeDensity.h"
#include "ParameterReader.h"

int main(int argc, char *argv[]) {
  try {
    smc::ParameterReader reader;
    reader.readFromFile("parameters.dat");
    reader.readFromArguments(argc, argv);
    smc::MakeDensity dens(&reader);
    const int nevent = (int)reader.getVal("nev", 50000);
    const int operation = (int)reader.getVal("operation", 9);
    const clock_t start = clock();
    switch (operation) {
      case 1: dens.generate_profile_ebe(nevent); break;
      case 2: dens.generate_profile_ebe_Jet(nevent); break;
      case 3: dens.generate_profile_average(nevent); break;
      case 9: dens.generateEccTable(nevent); break;
      default:
        std::printf("Error: operation choice %d not recognized.\n", operation);
        return 1;
    }
    std::printf("Time elapsed (in seconds): %g\n", (double)(clock() - start) / CLOCKS_PER_SEC);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "superMC (supermc_gb300): %s\n", e.what());
    return 1;
  }
  return 0;
}
