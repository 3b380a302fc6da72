// A host program written the way the reference's main.cpp drives FV::System2D (main.cpp:127-130),
// switched to the GPU path by including hteno.hpp.
// Usage: host_fv2d <result.dat> <state.bin> <initial.bin>
#include <cstdio>

#include "hteno.hpp"

using namespace hteno;

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  try {
    Options o;
    o.flux = HTENO_FLUX_HLLC;
    FV::System2D systemObj(0.0, 1.0, 64, 0.0, 1.0, 48, 0.4, 0.05, 0.0, 1.4, o);
    systemObj.Riemann2D();
    const std::vector<double> q0 = systemObj.state();
    FILE* f0 = std::fopen(argv[3], "wb");
    if (!f0) return 3;
    std::fwrite(q0.data(), sizeof(double), q0.size(), f0);
    std::fclose(f0);
    systemObj.timeStepping();
    systemObj.write(argv[1]);
    const std::vector<double> q = systemObj.state();
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 3;
    std::fwrite(q.data(), sizeof(double), q.size(), f);
    std::fclose(f);
    std::printf("t = %.17g\n", systemObj.time());
  } catch (const Error& e) {
    std::fprintf(stderr, "hteno error %d: %s\n", e.code, e.what());
    return 1;
  }
  return 0;
}
