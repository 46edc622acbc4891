// potential.h - host model of an AtomNN potential file and its device tables.
#pragma once
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "common.cuh"

namespace nnpgpu {

struct HBasisR {  // BasisR (src/nnp/basis_radial.hpp:53-94)
  int cut = 0, norm = 0, phi = 0;
  double rc = 0;
  std::vector<double> rs, eta;
};
struct HBasisA {  // BasisA (src/nnp/basis_angular.hpp:53-115)
  int cut = 0, norm = 0, phi = 0, alpha = 0;
  double rc = 0;
  std::vector<double> eta, zeta;
  std::vector<int> lam;
};
struct HNet {  // NN::ANN (src/ml/nn.hpp:218-341)
  int nin = 0, act = 0;
  std::string neuron;  // as written in the file
  std::vector<int> nodes;
  std::vector<double> inpw, inpb, outw, outb;
  std::vector<std::vector<double>> b, w;  // w[l] row-major [nodes[l]][cols]
};
struct HType {  // Type (src/nnp/type.hpp:22-94): name, mass, vacuum energy, other properties
  std::string name;
  double mass = 0, energy = 0;
  bool has_mass = false, has_energy = false;
  std::map<std::string, double> other;  // CHARGE, CHI, ETA, JS, C6, RVDW, RCOV when given
};
struct HPot {  // NNP (src/nnp/nnp.hpp:68-121)
  double rc = 0;
  int ntypes = 0;
  std::vector<HType> types;
  std::map<std::string, int> index;
  std::vector<std::vector<HBasisR>> rad;  // [I][J]
  std::vector<std::vector<HBasisA>> ang;  // [I][lidx(J,K)]
  std::vector<HNet> nets;
  std::vector<int> nin, ninR;
  std::vector<std::vector<int>> offR, offA;  // offsets (NNH::init_input, src/nnp/nnh.cpp:95-121)
};

struct PotError : std::runtime_error {
  int code;
  PotError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Parses the text format written by NNP::write (src/nnp/nnp.cpp:198-237); throws PotError.
HPot read_potential(const char* path);
// Writes it (NNP::write with Type::write, BasisR::write, BasisA::write and ANN::write: same
// tokens, order and number formats); throws PotError(NNPGPU_ERR_IO).
void write_potential(const HPot& pot, const char* path);
// Fills the kernel tables; throws PotError(NNPGPU_ERR_UNSUPPORTED) for forms the kernels lack.
void build_tables(const HPot& pot, PotParams& P, int& ne_max, int& nz_max);
// the per-block angular tables (AngP::tab) after build_tables: sets each block's tab offset and
// returns the floats; P.atab is set by the caller once they are on the device
std::vector<float> build_ang_tables(const HPot& pot, PotParams& P);

}  // namespace nnpgpu
