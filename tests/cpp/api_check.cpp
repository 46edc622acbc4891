// api_check - drives the C++ host surface (include/atomnn_gpu.hpp) the way the reference's
// compute tool drives AtomNN (src/nnp/nnpce.cpp:259-281) and prints every result, so that the
// test can compare them with the oracle.
//
// usage: api_check <potential> <POSCAR> <scratch binary file>
// prints: "nlist <atoms> <entries> <min entries>", "symm <i> <k> <value>" for atom 0,
//         "energy <E>", "cached <E>" (the networks on descriptors written to and read back from
//         a binary structure file), "positions <E>" (descriptors cleared: from the positions),
//         "compute <E without vacuum>", "force <i> <fx> <fy> <fz>", "batched <E>"
#include <cstdio>
#include <exception>
#include <vector>

#include "../../include/atomnn_gpu.hpp"

using namespace atomnn_gpu;

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  try {
    NNP nnp;
    NNP::read(argv[1], nnp);
    Structure struc;
    VASP::POSCAR::read(argv[2], struc);
    for (int n = 0; n < struc.nAtoms(); ++n) struc.type(n) = nnp.index(struc.name(n));
    NNP::init(nnp, struc);
    NeighborList nlist;
    nlist.build(struc, nnp.rc());
    long long entries = 0, mins = 0;
    for (int i = 0; i < nlist.size(); ++i)
      for (int j = 0; j < nlist.size(i); ++j) {
        ++entries;
        mins += nlist.neigh(i, j).min() ? 1 : 0;
      }
    std::printf("nlist %d %lld %lld\n", nlist.size(), entries, mins);
    NNP::symm(nnp, struc, nlist);
    for (size_t k = 0; k < struc.symm(0).size(); ++k) std::printf("symm 0 %zu %.9e\n", k, struc.symm(0)[k]);
    const double e = NNP::energy(nnp, struc);
    std::printf("energy %.10f\n", e);
    // the trainers' descriptor cache: the structure with its descriptors written to a binary
    // file, read back and evaluated without a neighbour list
    Structure::write_binary(struc, argv[3]);
    Structure back;
    Structure::read_binary(back, argv[3]);
    std::printf("cached %.10f\n", NNP::energy(nnp, back));
    for (int i = 0; i < back.nAtoms(); ++i) back.symm(i).clear();
    std::printf("positions %.10f\n", NNP::energy(nnp, back));
    NNP::force(nnp, struc, nlist);
    for (int i = 0; i < struc.nAtoms(); ++i)
      std::printf("force %d %.10f %.10f %.10f\n", i, struc.force(i)[0], struc.force(i)[1], struc.force(i)[2]);
    Structure copy = struc;
    NNP::compute(nnp, copy, nlist);
    std::printf("compute %.10f\n", copy.energy());
    std::vector<Structure> batch = {struc, struc};
    NNP::compute(nnp, batch, true);
    std::printf("batched %.10f %.10f\n", batch[0].energy(), batch[1].energy());
    // invalid input surfaces as the reference's exception type
    Structure bad = struc;
    bad.type(0) = 99;
    try {
      NNP::energy(nnp, bad);
      std::printf("invalid accepted\n");
    } catch (std::invalid_argument&) {
      std::printf("invalid_argument ok\n");
    }
  } catch (std::exception& ex) {
    std::printf("ERROR %s\n", ex.what());
    return 1;
  }
  return 0;
}
