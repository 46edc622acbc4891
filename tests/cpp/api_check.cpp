// api_check - drives the C++ host surface (include/atomnn_gpu.hpp) the way the reference's
// compute tool drives AtomNN (src/nnp/nnpce.cpp:259-281) and prints every result, so that the
// test can compare them with the oracle.
//
// usage: api_check <potential> <POSCAR> <scratch binary file>
// prints: "nlist <atoms> <entries> <min entries>", "symm <i> <k> <value>" for atom 0,
//         "energy <E>", "cached <E>" (the networks on descriptors written to and read back from
//         a binary structure file), "positions <E>" (descriptors cleared: from the positions),
//         "compute <E without vacuum>", "force <i> <fx> <fy> <fz>", "batched <E>", "trainer <E>" and
//         "tool <E> <f0x>" (the reference's trainer and compute-tool loops), "nbtype ok",
//         "r64 <j> <min> <rx> <ry> <rz> <dr>" for atom 0's list, "subset ok"
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
    // the trainer's loop (src/nnp/nnpte.cpp:1962-1977) and the compute tool's loop
    // (src/nnp/nnpce.cpp:259-281), with their own names and calls
    {
      std::vector<Structure> strucs(1, struc);
      for (int i = 0; i < (int)strucs.size(); ++i) NNP::init(nnp, strucs[i]);
      for (int i = 0; i < (int)strucs.size(); ++i) {
        NeighborList nlist(strucs[i], nnp.rc());
        NNP::symm(nnp, strucs[i], nlist);
      }
      std::printf("trainer %.10f\n", NNP::energy(nnp, strucs[0]));
      const bool force = true;
      std::vector<double> energy_nnp(strucs.size(), 0.0);
      for (int i = 0; i < (int)strucs.size(); ++i) {
        NeighborList nlist;
        nlist.build(strucs[i], nnp.rc());
        NNP::symm(nnp, strucs[i], nlist);
        NNP::energy(nnp, strucs[i]);
        if (force) NNP::force(nnp, strucs[i], nlist);
        energy_nnp[i] = strucs[i].energy();
      }
      std::printf("tool %.10f %.10f\n", energy_nnp[0], strucs[0].force(0)[0]);
    }
    // Neighbor::type, the FP64 vectors of atom 0, and the one-atom and subset builds
    {
      bool types = true;
      for (int i = 0; i < nlist.size(); ++i)
        for (int j = 0; j < nlist.size(i); ++j) types = types && nlist.neigh(i, j).type() == struc.type(nlist.neigh(i, j).index());
      std::printf("nbtype %s\n", types ? "ok" : "bad");
      for (int j = 0; j < nlist.size(0); ++j) {
        const Neighbor& nb = nlist.neigh(0, j);
        std::printf("r64 %d %d %.17g %.17g %.17g %.17g\n", nb.index(), nb.min() ? 1 : 0, nb.r()[0], nb.r()[1], nb.r()[2], nb.dr());
      }
      const int last = struc.nAtoms() - 1;
      NeighborList one;
      one.build(struc, nnp.rc(), last);
      NeighborList sub;
      sub.rc() = nnp.rc();
      sub.build(struc, std::vector<int>{0, last});
      bool same = one.size() == nlist.size() && one.size(0) == 0 && one.size(last) == nlist.size(last);
      same = same && sub.size(0) == nlist.size(0) && sub.size(last) == nlist.size(last) && (last < 2 || sub.size(1) == 0);
      for (int j = 0; same && j < nlist.size(last); ++j)
        same = one.neigh(last, j).index() == nlist.neigh(last, j).index() && one.neigh(last, j).min() == nlist.neigh(last, j).min() &&
               one.neigh(last, j).r()[0] == nlist.neigh(last, j).r()[0] && sub.neigh(last, j).dr() == nlist.neigh(last, j).dr();
      std::printf("subset %s\n", same ? "ok" : "bad");
    }
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
