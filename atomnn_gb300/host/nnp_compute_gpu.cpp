// nnp_compute_gpu - energies (and forces) of a set of structures with a potential, on the GPU.
//
// The GPU counterpart of the reference's compute tool (src/nnp/nnpce.cpp): the same parameter
// file (DATA, NNPOT, FORMAT, UNITS, FORCE, NORM; plus BF16 and BATCH), the same POSCAR/XYZ
// inputs and the same "energy <index> <reference> <nnp>" lines.  Instead of one MPI rank per
// group of structures and NeighborList::build + NNP::symm + NNP::energy + NNP::force per
// structure, every structure goes into batched evaluations of at most BATCH atoms.
//
// usage: nnp_compute_gpu <parameter file> [--dry-run]
//   --dry-run reads the parameters and every structure file and prints a summary without
//   touching the GPU.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "../../include/atomnn_gpu.hpp"

using namespace atomnn_gpu;

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <parameter file> [--dry-run]\n", argv[0]);
    return 1;
  }
  const bool dry = argc > 2 && std::strcmp(argv[2], "--dry-run") == 0;
  try {
    const auto t0 = std::chrono::steady_clock::now();
    const ComputeParams p = read_compute_params(argv[1]);
    std::printf("DATA   = \n");
    for (const std::string& d : p.data) std::printf("\t%s\n", d.c_str());
    std::printf("FORMAT = %s\nUNITS  = %s\nFORCE  = %d\nNORM   = %d\nBF16   = %d\nBATCH  = %lld\nNNPOT  = %s\n", p.format.c_str(),
                p.units.c_str(), (int)p.force, (int)p.norm, (int)p.bf16, p.batch_atoms, p.nnpot.c_str());
    // unit system of the readers (units::consts, METAL: Angstrom/eV; AU: Bohr/Hartree)
    const bool au = p.units == "AU";
    const double s_len = au ? 1.0 / 0.529177210903 : 1.0;
    const double s_energy = au ? 1.0 / 27.211386245988 : 1.0;

    const std::vector<std::string> files = read_data_lists(p.data);
    std::vector<Structure> strucs(files.size());
    long long total = 0;
    for (size_t i = 0; i < files.size(); ++i) {
      if (p.format == "POSCAR") VASP::POSCAR::read(files[i].c_str(), strucs[i], s_len);
      else XYZ::read(files[i].c_str(), strucs[i], s_len, s_energy);
      total += strucs[i].nAtoms();
    }
    std::printf("structures = %zu\natoms = %lld\n", strucs.size(), total);
    if (dry) {
      for (size_t i = 0; i < strucs.size(); ++i) {
        const Structure& s = strucs[i];
        std::printf("struc %zu %s natoms %d periodic %d energy %.10f first %s %.10f %.10f %.10f\n", i, files[i].c_str(), s.nAtoms(),
                    (int)s.periodic(), s.energy(), s.nAtoms() ? s.name(0).c_str() : "-", s.nAtoms() ? s.posn(0)[0] : 0.0,
                    s.nAtoms() ? s.posn(0)[1] : 0.0, s.nAtoms() ? s.posn(0)[2] : 0.0);
      }
      return 0;
    }

    NNP nnp;
    NNP::read(p.nnpot.c_str(), nnp);
    nnp.set_bf16(p.bf16);
    for (Structure& s : strucs)
      for (int n = 0; n < s.nAtoms(); ++n) {
        s.type(n) = nnp.index(s.name(n));
        if (s.type(n) < 0) throw std::invalid_argument("species " + s.name(n) + " is not in the potential");
      }
    std::vector<double> energy_ref(strucs.size());
    for (size_t i = 0; i < strucs.size(); ++i) energy_ref[i] = strucs[i].energy();

    // batched evaluations over consecutive structures of at most BATCH atoms each
    size_t b = 0;
    while (b < strucs.size()) {
      size_t e = b;
      long long atoms = 0;
      while (e < strucs.size() && (e == b || atoms + strucs[e].nAtoms() <= p.batch_atoms)) atoms += strucs[e++].nAtoms();
      std::vector<Structure> chunk(std::make_move_iterator(strucs.begin() + b), std::make_move_iterator(strucs.begin() + e));
      NNP::compute(nnp, chunk, p.force);
      std::move(chunk.begin(), chunk.end(), strucs.begin() + b);
      b = e;
    }

    for (size_t i = 0; i < strucs.size(); ++i) {
      if (!p.norm) std::printf("energy %zu %.6f %.6f\n", i, energy_ref[i], strucs[i].energy());
      else
        std::printf("energy/atom %zu %.6f %.6f\n", i, energy_ref[i] / strucs[i].nAtoms(), strucs[i].energy() / strucs[i].nAtoms());
    }
    if (p.force) {
      for (size_t i = 0; i < strucs.size(); ++i) {
        std::printf("struc[%zu]\n", i);
        for (int j = 0; j < strucs[i].nAtoms(); ++j)
          std::printf("force[%d] = %.10f %.10f %.10f\n", j, strucs[i].force(j)[0], strucs[i].force(j)[1], strucs[i].force(j)[2]);
      }
    }
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("time = %.6f\n", dt);
  } catch (std::exception& e) {
    std::printf("ERROR in nnp_compute_gpu:\n%s\n", e.what());
    return 1;
  }
  return 0;
}
