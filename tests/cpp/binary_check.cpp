// binary_check - reads a binary structure file with Structure::read_binary, prints what it
// holds and writes it back with Structure::write_binary (src/struc/structure.cpp:117-190), so
// that the test can compare both with an independent restatement of the layout.  No GPU use.
//
// usage: binary_check <in file> <out file>
// prints: "natoms <n>", "flags <16 digits>", "cell <9 values>", "state <8 values> <t>",
//         "atom <i> <name> <type> <index> <x> <y> <z> <fx> <fy> <fz> <symm size> <symm sum>",
//         "extra <i> <an> <mass> <charge> <radius> <chi> <eta> <c6> <js> <vx> <vy> <vz> <sx> <sy> <sz>"
//         (properties not flagged print as 0), or "ERROR <message>" and exit 1
#include <cstdio>
#include <exception>

#include "../../include/atomnn_gpu.hpp"

using namespace atomnn_gpu;

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  try {
    Structure s;
    Structure::read_binary(s, argv[1]);
    const AtomType& a = s.atomType();
    std::printf("natoms %d\nflags %d%d%d%d%d%d%d%d%d%d%d%d%d%d%d%d\n", s.nAtoms(), a.name, a.an, a.type, a.index, a.mass, a.charge, a.radius, a.chi,
                a.eta, a.c6, a.js, a.posn, a.vel, a.force, a.spin, a.symm);
    std::printf("cell");
    for (int k = 0; k < 9; ++k) std::printf(" %.17g", s.R()[k]);
    std::printf("\nstate %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %d\n", s.energy(), s.ewald(), s.temp(), s.press(), s.qtot(), s.pe(),
                s.ke(), s.dt(), s.t());
    for (int i = 0; i < s.nAtoms(); ++i) {
      double sum = 0.0;
      for (double g : s.symm(i)) sum += g;
      std::printf("atom %d %s %d %d %.17g %.17g %.17g %.17g %.17g %.17g %zu %.17g\n", i, s.name(i).empty() ? "-" : s.name(i).c_str(), s.type(i),
                  s.index(i), s.posn(i)[0], s.posn(i)[1], s.posn(i)[2], s.force(i)[0], s.force(i)[1], s.force(i)[2], s.symm(i).size(), sum);
      auto d = [&](std::vector<double>& v) { return v.empty() ? 0.0 : v[i]; };
      const Vec3d z;
      const Vec3d& v = s.vel().empty() ? z : s.vel(i);
      const Vec3d& sp = s.spin().empty() ? z : s.spin(i);
      std::printf("extra %d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", i,
                  s.an().empty() ? 0 : s.an(i), d(s.mass()), d(s.charge()), d(s.radius()), d(s.chi()), d(s.eta()), d(s.c6()), d(s.js()), v[0],
                  v[1], v[2], sp[0], sp[1], sp[2]);
    }
    Structure::write_binary(s, argv[2]);
  } catch (std::exception& ex) {
    std::printf("ERROR %s\n", ex.what());
    return 1;
  }
  return 0;
}
