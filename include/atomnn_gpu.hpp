// atomnn_gpu.hpp - C++ host surface of the GB300 engine for code written against AtomNN.
//
// The classes keep the names and call shapes of the reference's hot-path API so that a caller
// changes its includes and a using-declaration, not its calls:
//   NNP::read / init / symm / energy / force / compute   src/nnp/nnp.hpp:108-120
//   Structure (AtomData + Cell + State), AtomType        src/struc/structure.hpp:38-178,
//                                                        src/struc/atom_type.hpp:14-50
//   Structure::write_binary / read_binary                src/struc/structure.cpp:117-190
//   NeighborList::build, Neighbor                        src/struc/neighbor.hpp:28-85
//   VASP::POSCAR::read, XYZ::read                        src/format/vasp_struc.cpp:51-200,
//                                                        src/format/xyz_struc.cpp:38-130
// Everything is computed on the GPU through the C ABI of nnpgpu.h; this layer only converts
// between the reference's per-structure objects and the ABI's flat arrays, and turns non-zero
// status codes into the exceptions the reference throws (std::invalid_argument for bad input,
// std::runtime_error otherwise).
//
// Differences a caller should know:
//  * NNP::symm/energy/force/compute take the NeighborList argument for signature parity; the
//    GPU builds its own list at nnp.rc() (the same list NeighborList::build gives at that
//    cutoff).
//  * NNP::energy evaluates the networks on struc.symm() as the reference does, when every atom
//    holds a descriptor row of its type's input size (after NNP::symm, or read back from a
//    binary structure file); otherwise it computes the descriptors from the positions first.
//  * NNP::compute(nnp, std::vector<Structure>&, ...) evaluates many structures in one batched
//    launch sequence; it is the call the GPU is built for.
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "nnpgpu.h"

namespace atomnn_gpu {

// Three doubles with the element access of Eigen::Vector3d.
struct Vec3d {
  double v[3] = {0.0, 0.0, 0.0};
  Vec3d() = default;
  Vec3d(double x, double y, double z) : v{x, y, z} {}
  double& operator[](int k) { return v[k]; }
  const double& operator[](int k) const { return v[k]; }
  double& operator()(int k) { return v[k]; }
  const double& operator()(int k) const { return v[k]; }
  double* data() { return v; }
  const double* data() const { return v; }
};

// Which per-atom properties a structure carries (AtomType, src/struc/atom_type.hpp:14-50).  name,
// type, index, posn, force and symm are always allocated here; the flags say which of them a
// binary structure file holds, and which of the other properties are allocated.
struct AtomType {
  bool frac = false;
  bool name = true, an = false, type = true, index = true;
  bool mass = false, charge = false, radius = false, chi = false, eta = false, c6 = false, js = false;
  bool posn = true, vel = false, force = true, spin = false;
  bool symm = true;
};

// One structure: per-atom data (AtomData), the lattice (Cell) and the scalar state (State).
class Structure {
 public:
  Structure() = default;
  explicit Structure(int nAtoms) { resize(nAtoms); }
  Structure(int nAtoms, const AtomType& atomT) { resize(nAtoms, atomT); }

  void resize(int nAtoms);
  void resize(int nAtoms, const AtomType& atomT);
  void clear();
  int nAtoms() const { return nAtoms_; }
  const AtomType& atomType() const { return atomT_; }

  // lattice (Cell::init, src/struc/cell.cpp:45-70): lv column-major, columns = lattice vectors;
  // an all-zero lattice means a non-periodic structure
  void init(const double lv[9]);
  const std::array<double, 9>& R() const { return R_; }
  double R(int row, int col) const { return R_[3 * col + row]; }
  bool periodic() const;

  // per-atom data (AtomData)
  std::vector<std::string>& name() { return name_; }
  const std::vector<std::string>& name() const { return name_; }
  std::string& name(int i) { return name_[i]; }
  const std::string& name(int i) const { return name_[i]; }
  std::vector<int>& type() { return type_; }
  const std::vector<int>& type() const { return type_; }
  int& type(int i) { return type_[i]; }
  const int& type(int i) const { return type_[i]; }
  std::vector<int>& index() { return index_; }
  const std::vector<int>& index() const { return index_; }
  int& index(int i) { return index_[i]; }
  const int& index(int i) const { return index_[i]; }
  std::vector<Vec3d>& posn() { return posn_; }
  const std::vector<Vec3d>& posn() const { return posn_; }
  Vec3d& posn(int i) { return posn_[i]; }
  const Vec3d& posn(int i) const { return posn_[i]; }
  std::vector<Vec3d>& force() { return force_; }
  const std::vector<Vec3d>& force() const { return force_; }
  Vec3d& force(int i) { return force_[i]; }
  const Vec3d& force(int i) const { return force_[i]; }
  std::vector<std::vector<double>>& symm() { return symm_; }
  const std::vector<std::vector<double>>& symm() const { return symm_; }
  std::vector<double>& symm(int i) { return symm_[i]; }
  const std::vector<double>& symm(int i) const { return symm_[i]; }

  // properties allocated when the AtomType flag is set (empty otherwise)
  std::vector<int>& an() { return an_; }
  int& an(int i) { return an_[i]; }
  std::vector<double>& mass() { return mass_; }
  double& mass(int i) { return mass_[i]; }
  std::vector<double>& charge() { return charge_; }
  double& charge(int i) { return charge_[i]; }
  std::vector<double>& radius() { return radius_; }
  double& radius(int i) { return radius_[i]; }
  std::vector<double>& chi() { return chi_; }
  double& chi(int i) { return chi_[i]; }
  std::vector<double>& eta() { return eta_; }
  double& eta(int i) { return eta_[i]; }
  std::vector<double>& c6() { return c6_; }
  double& c6(int i) { return c6_[i]; }
  std::vector<double>& js() { return js_; }
  double& js(int i) { return js_[i]; }
  std::vector<Vec3d>& vel() { return vel_; }
  Vec3d& vel(int i) { return vel_[i]; }
  std::vector<Vec3d>& spin() { return spin_; }
  Vec3d& spin(int i) { return spin_[i]; }

  // State (src/struc/state.hpp)
  double& energy() { return energy_; }
  const double& energy() const { return energy_; }
  double& ewald() { return ewald_; }
  double& temp() { return temp_; }
  double& press() { return press_; }
  double& qtot() { return qtot_; }
  double& pe() { return pe_; }
  double& ke() { return ke_; }
  double& dt() { return dt_; }
  int& t() { return t_; }

  // Structure::write_binary / read_binary (src/struc/structure.cpp:117-190): the reference's
  // byte layout (an int byte count, then the lattice, the state and the per-atom data the
  // AtomType flags select), so files pass between the two codes.  Throw std::runtime_error on
  // IO errors and on a malformed file.
  static void write_binary(const Structure& struc, const char* file);
  static void read_binary(Structure& struc, const char* file);

 private:
  friend struct BinaryIO;
  int nAtoms_ = 0;
  AtomType atomT_;
  std::array<double, 9> R_{};
  std::vector<std::string> name_;
  std::vector<int> type_, index_, an_;
  std::vector<double> mass_, charge_, radius_, chi_, eta_, c6_, js_;
  std::vector<Vec3d> posn_, force_, vel_, spin_;
  std::vector<std::vector<double>> symm_;
  double energy_ = 0.0, ewald_ = 0.0, temp_ = 0.0, press_ = 0.0, qtot_ = 0.0, pe_ = 0.0, ke_ = 0.0, dt_ = 0.0;
  int t_ = 0;
};

// One entry of a neighbour list (Neighbor, src/struc/neighbor.hpp:28-54): r points from the
// neighbour's image to the centre, dr is its length, type the neighbour's type (struc.type(j)),
// cell the image's integer lattice translation.
class Neighbor {
 public:
  int& index() { return index_; }
  const int& index() const { return index_; }
  int& type() { return type_; }
  const int& type() const { return type_; }
  Vec3d& r() { return r_; }
  const Vec3d& r() const { return r_; }
  double& dr() { return dr_; }
  const double& dr() const { return dr_; }
  bool& min() { return min_; }
  const bool& min() const { return min_; }
  std::array<int, 3>& cell() { return cell_; }
  const std::array<int, 3>& cell() const { return cell_; }

 private:
  int index_ = 0;
  int type_ = -1;
  Vec3d r_;
  double dr_ = 0.0;
  bool min_ = false;
  std::array<int, 3> cell_{};
};

class NNP;

// Neighbour lists of one structure, built on the GPU (NeighborList::build,
// src/struc/neighbor.cpp:59-171): same entries, order and minimum-image flags.  Vectors and
// distances are FP64: r = posn(i) - posn(j) - R * cell, recomputed on the host from the image's
// lattice translation.  Entries of a periodic structure carry struc.index(j) as their index (j
// in a non-periodic one), as the reference's build does.
class NeighborList {
 public:
  NeighborList() = default;
  // NeighborList(const Structure&, double) (src/struc/neighbor.hpp:71): builds at once
  NeighborList(const Structure& struc, double rc) { build(struc, rc); }
  // builds with the device context of the most recently read NNP (the reference's build has
  // no potential argument); throws std::runtime_error when no NNP has been read
  void build(const Structure& struc, double rc);
  void build(const NNP& nnp, const Structure& struc, double rc);
  // build(struc, rc, ii) and build(struc, rc, subset) (src/struc/neighbor.cpp:173-394): the list
  // is resized to the structure's atoms and only atom ii's (the subset's) lists are rebuilt; the
  // others keep their entries.  The overloads without rc use the list's last cutoff.
  void build(const Structure& struc, double rc, int ii);
  void build(const Structure& struc, double rc, const std::vector<int>& subset);
  void build(const Structure& struc) { build(struc, rc_); }
  void build(const Structure& struc, int ii) { build(struc, rc_, ii); }
  void build(const Structure& struc, const std::vector<int>& subset) { build(struc, rc_, subset); }
  void clear() {
    rc_ = 0.0;
    neigh_.clear();
  }
  double& rc() { return rc_; }
  const double& rc() const { return rc_; }
  int size() const { return (int)neigh_.size(); }
  int size(int i) const { return (int)neigh_[i].size(); }
  std::vector<Neighbor>& neigh(int i) { return neigh_[i]; }
  const std::vector<Neighbor>& neigh(int i) const { return neigh_[i]; }
  Neighbor& neigh(int i, int j) { return neigh_[i][j]; }
  const Neighbor& neigh(int i, int j) const { return neigh_[i][j]; }

 private:
  // lists of the atoms in subset (every atom when all is set) into neigh_
  void build_atoms(const NNP& nnp, const Structure& struc, double rc, const std::vector<int>& subset, bool all);
  double rc_ = 0.0;
  std::vector<std::vector<Neighbor>> neigh_;
};

// The potential: one engine context (device, stream, weights) behind the reference's static API.
class NNP {
 public:
  NNP() = default;

  int ntypes() const;
  int index(const char* name) const;
  int index(const std::string& name) const { return index(name.c_str()); }
  double rc() const;
  int nInput(int type) const;
  const std::string& file() const { return file_; }
  nnpgpu_ctx* ctx() const { return ctx_.get(); }
  bool bf16() const { return bf16_; }
  void set_bf16(bool on) { bf16_ = on; }  // tensor-core networks for every later call

  // NNP::read(const char*, NNP&) (src/nnp/nnp.cpp:182-191,244-308); opts may be null
  static void read(const char* file, NNP& nnp, const nnpgpu_opts* opts = nullptr);
  // NNP::write(const char*, const NNP&) (src/nnp/nnp.cpp:198-237): the potential with the
  // networks' current parameters (as set through nnpgpu_set_params by a trainer)
  static void write(const char* file, const NNP& nnp);
  // NNP::init: sizes struc.symm(i) to the input size of atom i's type
  static void init(const NNP& nnp, Structure& struc);
  // NNP::symm: struc.symm(i) for every atom (nnp.cpp:334-381)
  static void symm(NNP& nnp, Structure& struc, const NeighborList& nlist);
  // NNP::energy: sum of atomic energies including each species' vacuum energy (nnp.cpp:390-402),
  // the networks evaluated on struc.symm() (from the positions when symm is not filled); sets
  // struc.energy() and returns it
  static double energy(NNP& nnp, Structure& struc);
  // NNP::force: struc.force(i) (nnp.cpp:416-482)
  static void force(NNP& nnp, Structure& struc, const NeighborList& nlist);
  // NNP::compute: energy without the vacuum energies, and forces (nnp.cpp:496-566)
  static void compute(NNP& nnp, Structure& struc, const NeighborList& nlist);
  // batched: energies (struc.energy(), vacuum energies included unless no_vacuum) and, when
  // force is set, forces of all structures in one evaluation; atom types come from
  // struc.type(), which the caller sets with nnp.index(name) as the reference's tools do
  static void compute(NNP& nnp, std::vector<Structure>& strucs, bool force, bool no_vacuum = false);

 private:
  std::shared_ptr<nnpgpu_ctx> ctx_;
  std::string file_;
  bool bf16_ = false;
  friend class NeighborList;
};

// File readers with the reference's parsing rules.  s_len converts the file's length unit to
// the run's (1 for METAL units, Bohr per Angstrom for AU); s_energy likewise for energies.
namespace VASP {
namespace POSCAR {
void read(const char* file, Structure& struc, double s_len = 1.0);
}  // namespace POSCAR
}  // namespace VASP
namespace XYZ {
void read(const char* file, Structure& struc, double s_len = 1.0, double s_energy = 1.0);
}  // namespace XYZ

// Parameter file of the compute tool (src/nnp/nnpce.cpp:146-166): DATA (repeatable), NNPOT,
// FORMAT, UNITS, FORCE, NORM; plus BF16 (tensor-core networks) and BATCH (atoms per batched
// evaluation) for the GPU.  Keys are case-insensitive; '#' starts a comment.
struct ComputeParams {
  std::vector<std::string> data;
  std::string nnpot;
  std::string format = "POSCAR";
  std::string units = "METAL";
  bool force = false;
  bool norm = false;
  bool bf16 = false;
  long long batch_atoms = 4000000;
};
ComputeParams read_compute_params(const char* file);
// string::boolean of the reference (src/str/string.cpp:177-187): true for "T", "t", "TRUE",
// "true", "True" and "1", false for anything else
bool boolean(const std::string& s);
// the list of structure files named by the DATA files, one per non-empty line
std::vector<std::string> read_data_lists(const std::vector<std::string>& data);

}  // namespace atomnn_gpu
