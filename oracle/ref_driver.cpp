// ref_driver.cpp - runs the reference's own NNP energy/force path (markdellostritto/AtomNN
// sources, compiled unchanged by oracle/Makefile.ref against the Eigen-API shim in
// oracle/ref_shim/) on structures given in a text file, and prints every intermediate the
// oracle restates.
//
// TEST INFRASTRUCTURE ONLY: it pins the FP64 oracle (oracle/nnp_oracle.cpp) to the reference;
// the engine never links or runs it.  The calls follow the compute tool's loop
// (src/nnp/nnpce.cpp:248-281): NNP::read, types from the species names (NNP::index), NNP::init,
// NeighborList::build(struc, rc), NNP::symm, NNP::energy, NNP::force; then NNP::compute on the
// same list for the energy without vacuum energies (src/nnp/nnp.cpp:496-566).
//
// Input (argv[1]):  line 1 the potential file; line 2 the number of structures; per structure
//   "natoms periodic", if periodic one line of the 9 lattice entries R(0,0) R(1,0) R(2,0) R(0,1)
//   ... (columns = lattice vectors), then natoms lines "name x y z".
// Output (stdout), per structure:
//   struc k natoms
//   energy E           (NNP::energy after NNP::symm, vacuum energies included)
//   energy_compute E   (NNP::compute)
//   f i fx fy fz       (NNP::force)
//   fc i fx fy fz      (NNP::compute)
//   g i n g_0 ... g_{n-1}
//   nb i count         followed by count lines "j type min dr rx ry rz"
// Flags (argv[2], optional): "nolist" omits the neighbour lists.
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "src/nnp/nnp.hpp"
#include "src/struc/neighbor.hpp"
#include "src/struc/structure.hpp"

static void run(NNP& nnp, Structure& struc, int k, bool lists) {
  const int n = struc.nAtoms();
  for (int i = 0; i < n; ++i) {
    struc.index(i) = i;
    struc.type(i) = nnp.index(struc.name(i));
  }
  NNP::init(nnp, struc);
  NeighborList nlist;
  nlist.build(struc, nnp.rc());
  NNP::symm(nnp, struc, nlist);
  const double e = NNP::energy(nnp, struc);
  NNP::force(nnp, struc, nlist);
  std::vector<Eigen::Vector3d> f(n);
  for (int i = 0; i < n; ++i) f[i] = struc.force(i);
  NNP::compute(nnp, struc, nlist);
  const double ec = struc.energy();
  std::printf("struc %d %d\nenergy %.17g\nenergy_compute %.17g\n", k, n, e, ec);
  for (int i = 0; i < n; ++i) std::printf("f %d %.17g %.17g %.17g\n", i, f[i][0], f[i][1], f[i][2]);
  for (int i = 0; i < n; ++i)
    std::printf("fc %d %.17g %.17g %.17g\n", i, struc.force(i)[0], struc.force(i)[1], struc.force(i)[2]);
  for (int i = 0; i < n; ++i) {
    const int m = (int)struc.symm(i).size();
    std::printf("g %d %d", i, m);
    for (int q = 0; q < m; ++q) std::printf(" %.17g", struc.symm(i)[q]);
    std::printf("\n");
  }
  if (!lists) return;
  for (int i = 0; i < n; ++i) {
    std::printf("nb %d %d\n", i, nlist.size(i));
    for (int j = 0; j < nlist.size(i); ++j) {
      const Neighbor& nb = nlist.neigh(i, j);
      std::printf("%d %d %d %.17g %.17g %.17g %.17g\n", nb.index(), nb.type(), nb.min() ? 1 : 0, nb.dr(), nb.r()[0], nb.r()[1],
                  nb.r()[2]);
    }
  }
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s input.txt [nolist]\n", argv[0]);
    return 2;
  }
  const bool lists = !(argc > 2 && std::string(argv[2]) == "nolist");
  try {
    std::ifstream in(argv[1]);
    if (!in) throw std::runtime_error(std::string("cannot open ") + argv[1]);
    std::string potfile;
    std::getline(in, potfile);
    int nstruc = 0;
    in >> nstruc;
    NNP nnp;
    NNP::read(potfile.c_str(), nnp);
    AtomType atomT;
    atomT.name = true;
    atomT.an = false;
    atomT.type = true;
    atomT.index = true;
    atomT.posn = true;
    atomT.force = true;
    atomT.symm = true;
    for (int k = 0; k < nstruc; ++k) {
      int n = 0, periodic = 0;
      in >> n >> periodic;
      Structure struc(n, atomT);
      if (periodic) {
        Eigen::Matrix3d R;
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) in >> R(r, c);
        static_cast<Cell&>(struc).init(R);
      }
      for (int i = 0; i < n; ++i) {
        std::string name;
        double x, y, z;
        in >> name >> x >> y >> z;
        struc.name(i) = name;
        struc.posn(i) = Eigen::Vector3d(x, y, z);
      }
      if (!in) throw std::runtime_error("truncated input");
      run(nnp, struc, k, lists);
    }
  } catch (std::exception& e) {
    std::fprintf(stderr, "ref_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
