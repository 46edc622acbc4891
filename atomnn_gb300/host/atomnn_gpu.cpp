// atomnn_gpu.cpp - the C++ host surface (include/atomnn_gpu.hpp) over the C ABI (nnpgpu.h).
#include "../../include/atomnn_gpu.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>

namespace atomnn_gpu {

namespace {

// Status code -> the exception the reference throws for the same failure.
[[noreturn]] void fail(nnpgpu_ctx* ctx, int code, const char* where) {
  const std::string msg = std::string(where) + ": " + (ctx ? nnpgpu_last_error(ctx) : "no context");
  if (code == NNPGPU_ERR_INVALID) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

void check(nnpgpu_ctx* ctx, int code, const char* where) {
  if (code != NNPGPU_OK) fail(ctx, code, where);
}

// The context of the most recently read potential, for NeighborList::build(struc, rc).
std::mutex g_last_mu;
std::weak_ptr<nnpgpu_ctx> g_last;

std::string upper(std::string s) {
  for (char& ch : s) ch = (char)std::toupper((unsigned char)ch);
  return s;
}

// whitespace tokens of a line after removing a '#' comment
std::vector<std::string> tokens(const std::string& line) {
  std::string s = line.substr(0, line.find('#'));
  std::istringstream in(s);
  std::vector<std::string> out;
  std::string t;
  while (in >> t) out.push_back(t);
  return out;
}

struct Flat {
  std::vector<int> natoms, species;
  std::vector<double> posn, cell;
};

void flatten(const NNP& nnp, const Structure* const* strucs, int n, Flat& f) {
  f.natoms.resize(n);
  f.cell.resize(9 * (size_t)n);
  size_t tot = 0;
  for (int s = 0; s < n; ++s) tot += (size_t)strucs[s]->nAtoms();
  f.posn.resize(3 * tot);
  f.species.resize(tot);
  size_t a = 0;
  for (int s = 0; s < n; ++s) {
    const Structure& st = *strucs[s];
    f.natoms[s] = st.nAtoms();
    for (int k = 0; k < 9; ++k) f.cell[9 * (size_t)s + k] = st.R()[k];
    for (int i = 0; i < st.nAtoms(); ++i, ++a) {
      for (int x = 0; x < 3; ++x) f.posn[3 * a + x] = st.posn(i)[x];
      const int t = st.type(i);
      if (t < 0 || t >= nnp.ntypes())
        throw std::invalid_argument("atom " + std::to_string(i) + " has type " + std::to_string(t) +
                                    ", not a type of the potential (set struc.type(i) = nnp.index(name))");
      f.species[a] = t;
    }
  }
}

int max_input(const NNP& nnp) {
  int m = 0;
  for (int t = 0; t < nnp.ntypes(); ++t) m = std::max(m, nnp.nInput(t));
  return m;
}

}  // namespace

// ------------------------------------------------------------------------------ Structure
void Structure::resize(int nAtoms) { resize(nAtoms, atomT_); }

void Structure::resize(int nAtoms, const AtomType& atomT) {
  if (nAtoms < 0) throw std::invalid_argument("Structure::resize: negative atom count");
  nAtoms_ = nAtoms;
  atomT_ = atomT;
  name_.resize(nAtoms);
  type_.resize(nAtoms, -1);
  index_.resize(nAtoms);
  for (int i = 0; i < nAtoms; ++i) index_[i] = i;
  posn_.resize(nAtoms);
  force_.resize(nAtoms);
  symm_.resize(nAtoms);
  auto opt = [&](auto& v, bool on) { v.resize(on ? nAtoms : 0); };
  opt(an_, atomT.an);
  opt(mass_, atomT.mass);
  opt(charge_, atomT.charge);
  opt(radius_, atomT.radius);
  opt(chi_, atomT.chi);
  opt(eta_, atomT.eta);
  opt(c6_, atomT.c6);
  opt(js_, atomT.js);
  opt(vel_, atomT.vel);
  opt(spin_, atomT.spin);
}

void Structure::clear() {
  *this = Structure();
}

void Structure::init(const double lv[9]) {
  for (int k = 0; k < 9; ++k) R_[k] = lv[k];
}

bool Structure::periodic() const {
  for (double v : R_)
    if (v != 0.0) return true;
  return false;
}

// ------------------------------------------------------------------------------ binary files
// The byte layout of serialize::pack for Structure (src/struc/structure.cpp:604-649, its parts in
// src/struc/cell.cpp:182-206, src/struc/state.cpp:48-103, src/struc/atom_type.cpp:95-180,
// src/mem/serialize.cpp:21-180 and src/math/eigen.cpp:40-160), native byte order:
//   Cell      R, 9 doubles column-major
//   State     energy ewald temp press qtot pe ke dt (doubles), t (int)
//   AtomData  16 one-byte flags (name an type index mass charge radius chi eta c6 js posn vel
//             force spin symm), int natoms, then each flagged property in that order:
//             strings as int count + (int length + chars) each, int/double arrays as int count +
//             values, 3-vectors as int count + 3 doubles each, symm as int count + (int size +
//             doubles) per atom.
// A file is an int byte count followed by those bytes.
struct BinaryIO {
  std::vector<char> buf;
  size_t pos = 0;

  template <class T>
  void put(const T& v) {
    const char* b = reinterpret_cast<const char*>(&v);
    buf.insert(buf.end(), b, b + sizeof(T));
  }
  void put_bytes(const void* p, size_t n) {
    const char* b = static_cast<const char*>(p);
    buf.insert(buf.end(), b, b + n);
  }
  template <class T>
  void put_vec(const std::vector<T>& v) {
    put((int)v.size());
    if (!v.empty()) put_bytes(v.data(), sizeof(T) * v.size());
  }
  void put_vec3(const std::vector<Vec3d>& v) {
    put((int)v.size());
    for (const Vec3d& x : v) put_bytes(x.data(), 3 * sizeof(double));
  }
  template <class T>
  T get() {
    T v;
    get_bytes(&v, sizeof(T));
    return v;
  }
  void get_bytes(void* p, size_t n) {
    if (n > buf.size() - pos) throw std::runtime_error("read_binary: file ends inside a record");
    std::memcpy(p, buf.data() + pos, n);
    pos += n;
  }
  int get_count(size_t elem) {
    const int n = get<int>();
    if (n < 0 || (elem > 0 && (size_t)n > (buf.size() - pos) / elem)) throw std::runtime_error("read_binary: invalid element count");
    return n;
  }
  template <class T>
  void get_vec(std::vector<T>& v) {
    v.resize(get_count(sizeof(T)));
    if (!v.empty()) get_bytes(v.data(), sizeof(T) * v.size());
  }
  void get_vec3(std::vector<Vec3d>& v) {
    v.resize(get_count(3 * sizeof(double)));
    for (Vec3d& x : v) get_bytes(x.data(), 3 * sizeof(double));
  }

  static void pack(const Structure& s, BinaryIO& o) {
    o.put_bytes(s.R_.data(), 9 * sizeof(double));
    for (double v : {s.energy_, s.ewald_, s.temp_, s.press_, s.qtot_, s.pe_, s.ke_, s.dt_}) o.put(v);
    o.put(s.t_);
    const AtomType& a = s.atomT_;
    for (bool f : {a.name, a.an, a.type, a.index, a.mass, a.charge, a.radius, a.chi, a.eta, a.c6, a.js, a.posn, a.vel, a.force, a.spin, a.symm})
      o.put((char)(f ? 1 : 0));
    o.put(s.nAtoms_);
    if (a.name) {
      o.put((int)s.name_.size());
      for (const std::string& n : s.name_) {
        o.put((int)n.size());
        o.put_bytes(n.data(), n.size());
      }
    }
    if (a.an) o.put_vec(s.an_);
    if (a.type) o.put_vec(s.type_);
    if (a.index) o.put_vec(s.index_);
    if (a.mass) o.put_vec(s.mass_);
    if (a.charge) o.put_vec(s.charge_);
    if (a.radius) o.put_vec(s.radius_);
    if (a.chi) o.put_vec(s.chi_);
    if (a.eta) o.put_vec(s.eta_);
    if (a.c6) o.put_vec(s.c6_);
    if (a.js) o.put_vec(s.js_);
    if (a.posn) o.put_vec3(s.posn_);
    if (a.vel) o.put_vec3(s.vel_);
    if (a.force) o.put_vec3(s.force_);
    if (a.spin) o.put_vec3(s.spin_);
    if (a.symm) {
      o.put((int)s.symm_.size());
      for (const std::vector<double>& g : s.symm_) o.put_vec(g);
    }
  }

  static void unpack(Structure& s, BinaryIO& in) {
    std::array<double, 9> R;
    in.get_bytes(R.data(), 9 * sizeof(double));
    double st[8];
    for (double& v : st) v = in.get<double>();
    const int t = in.get<int>();
    AtomType a;
    bool* flags[16] = {&a.name, &a.an, &a.type, &a.index, &a.mass, &a.charge, &a.radius, &a.chi,
                       &a.eta, &a.c6, &a.js, &a.posn, &a.vel, &a.force, &a.spin, &a.symm};
    for (bool* f : flags) *f = in.get<char>() != 0;
    const int n = in.get<int>();
    if (n < 0) throw std::runtime_error("read_binary: negative atom count");
    Structure r;
    r.resize(n, a);
    r.R_ = R;
    r.energy_ = st[0]; r.ewald_ = st[1]; r.temp_ = st[2]; r.press_ = st[3];
    r.qtot_ = st[4]; r.pe_ = st[5]; r.ke_ = st[6]; r.dt_ = st[7];
    r.t_ = t;
    // each array must hold one entry per atom (AtomData::resize sizes them so in the reference)
    auto need = [n](size_t got) {
      if ((int)got != n) throw std::runtime_error("read_binary: per-atom array does not match the atom count");
    };
    if (a.name) {
      r.name_.resize(in.get_count(sizeof(int)));
      need(r.name_.size());
      for (std::string& nm : r.name_) {
        nm.resize(in.get_count(1));
        if (!nm.empty()) in.get_bytes(&nm[0], nm.size());
      }
    }
    if (a.an) { in.get_vec(r.an_); need(r.an_.size()); }
    if (a.type) { in.get_vec(r.type_); need(r.type_.size()); }
    if (a.index) { in.get_vec(r.index_); need(r.index_.size()); }
    if (a.mass) { in.get_vec(r.mass_); need(r.mass_.size()); }
    if (a.charge) { in.get_vec(r.charge_); need(r.charge_.size()); }
    if (a.radius) { in.get_vec(r.radius_); need(r.radius_.size()); }
    if (a.chi) { in.get_vec(r.chi_); need(r.chi_.size()); }
    if (a.eta) { in.get_vec(r.eta_); need(r.eta_.size()); }
    if (a.c6) { in.get_vec(r.c6_); need(r.c6_.size()); }
    if (a.js) { in.get_vec(r.js_); need(r.js_.size()); }
    if (a.posn) { in.get_vec3(r.posn_); need(r.posn_.size()); }
    if (a.vel) { in.get_vec3(r.vel_); need(r.vel_.size()); }
    if (a.force) { in.get_vec3(r.force_); need(r.force_.size()); }
    if (a.spin) { in.get_vec3(r.spin_); need(r.spin_.size()); }
    if (a.symm) {
      r.symm_.resize(in.get_count(sizeof(int)));
      need(r.symm_.size());
      for (std::vector<double>& g : r.symm_) in.get_vec(g);
    }
    if (in.pos != in.buf.size()) throw std::runtime_error("read_binary: trailing bytes after the structure");
    s = std::move(r);
  }
};

void Structure::write_binary(const Structure& struc, const char* file) {
  BinaryIO o;
  BinaryIO::pack(struc, o);
  std::FILE* f = std::fopen(file, "wb");
  if (!f) throw std::runtime_error(std::string("write_binary(Structure&,const char*): Could not open file: ") + file);
  const int nbytes = (int)o.buf.size();
  const bool ok = std::fwrite(&nbytes, sizeof(int), 1, f) == 1 && std::fwrite(o.buf.data(), 1, o.buf.size(), f) == o.buf.size();
  const bool closed = std::fclose(f) == 0;
  if (!ok || !closed) throw std::runtime_error(std::string("write_binary(Structure&,const char*): Write error: ") + file);
}

void Structure::read_binary(Structure& struc, const char* file) {
  std::FILE* f = std::fopen(file, "rb");
  if (!f) throw std::runtime_error(std::string("read_binary(Structure&,const char*): Could not open file: ") + file);
  BinaryIO in;
  int nbytes = 0;
  bool ok = std::fread(&nbytes, sizeof(int), 1, f) == 1 && nbytes >= 0;
  if (ok) {
    in.buf.resize((size_t)nbytes);
    ok = std::fread(in.buf.data(), 1, in.buf.size(), f) == in.buf.size();
  }
  std::fclose(f);
  if (!ok) throw std::runtime_error(std::string("read_binary(Structure&,const char*): Read error: ") + file);
  BinaryIO::unpack(struc, in);
}

// ------------------------------------------------------------------------------ NNP
int NNP::ntypes() const { return ctx_ ? nnpgpu_ntypes(ctx_.get()) : 0; }
int NNP::index(const char* name) const { return ctx_ ? nnpgpu_type_index(ctx_.get(), name) : -1; }
double NNP::rc() const { return ctx_ ? nnpgpu_cutoff(ctx_.get()) : 0.0; }
int NNP::nInput(int type) const { return ctx_ ? nnpgpu_ninput(ctx_.get(), type) : -1; }

void NNP::read(const char* file, NNP& nnp, const nnpgpu_opts* opts) {
  if (!file) throw std::invalid_argument("NNP::read: no file");
  nnpgpu_ctx* c = nullptr;
  const int code = nnpgpu_create(file, opts, &c);
  std::shared_ptr<nnpgpu_ctx> holder(c, [](nnpgpu_ctx* p) { nnpgpu_destroy(p); });
  if (code != NNPGPU_OK) fail(c, code, "NNP::read");
  nnp.ctx_ = holder;
  nnp.file_ = file;
  std::lock_guard<std::mutex> l(g_last_mu);
  g_last = holder;
}

void NNP::write(const char* file, const NNP& nnp) {
  if (!nnp.ctx_) throw std::runtime_error("NNP::write: no potential read");
  if (!file) throw std::invalid_argument("NNP::write: no file");
  check(nnp.ctx(), nnpgpu_write_potential(nnp.ctx(), file), "NNP::write");
}

void NNP::init(const NNP& nnp, Structure& struc) {
  for (int i = 0; i < struc.nAtoms(); ++i) {
    const int t = struc.type(i);
    if (t < 0 || t >= nnp.ntypes()) throw std::invalid_argument("NNP::init: atom type not in the potential");
    struc.symm(i).assign(nnp.nInput(t), 0.0);
  }
}

void NNP::symm(NNP& nnp, Structure& struc, const NeighborList&) {
  if (!nnp.ctx_) throw std::runtime_error("NNP::symm: no potential read");
  const Structure* p = &struc;
  Flat f;
  flatten(nnp, &p, 1, f);
  const int stride = max_input(nnp);
  std::vector<float> G((size_t)std::max(struc.nAtoms(), 1) * stride);
  check(nnp.ctx(), nnpgpu_compute(nnp.ctx(), 1, f.natoms.data(), f.posn.data(), f.species.data(), f.cell.data(), NNPGPU_SYMM, nullptr,
                                  nullptr, G.data()),
        "NNP::symm");
  for (int i = 0; i < struc.nAtoms(); ++i) {
    const int nin = nnp.nInput(struc.type(i));
    struc.symm(i).resize(nin);
    for (int k = 0; k < nin; ++k) struc.symm(i)[k] = G[(size_t)i * stride + k];
  }
}

double NNP::energy(NNP& nnp, Structure& struc) {
  if (!nnp.ctx_) throw std::runtime_error("NNP::energy: no potential read");
  const int n = struc.nAtoms();
  bool filled = n > 0;
  for (int i = 0; i < n && filled; ++i) {
    const int t = struc.type(i);
    if (t < 0 || t >= nnp.ntypes()) throw std::invalid_argument("NNP::energy: atom type not in the potential");
    filled = (int)struc.symm(i).size() == nnp.nInput(t);
  }
  if (filled) {  // the reference's path: the networks on the stored descriptors
    const int stride = max_input(nnp);
    std::vector<double> G((size_t)n * stride, 0.0);
    for (int i = 0; i < n; ++i) std::copy(struc.symm(i).begin(), struc.symm(i).end(), G.begin() + (size_t)i * stride);
    double e = 0.0;
    check(nnp.ctx(), nnpgpu_energy_symm(nnp.ctx(), 1, &n, struc.type().data(), G.data(), stride, nnp.bf16_ ? NNPGPU_BF16 : 0, &e),
          "NNP::energy");
    struc.energy() = e;
    return e;
  }
  const Structure* p = &struc;
  Flat f;
  flatten(nnp, &p, 1, f);
  double e = 0.0;
  const int flags = NNPGPU_ENERGY | (nnp.bf16_ ? NNPGPU_BF16 : 0);
  check(nnp.ctx(), nnpgpu_compute(nnp.ctx(), 1, f.natoms.data(), f.posn.data(), f.species.data(), f.cell.data(), flags, &e, nullptr, nullptr),
        "NNP::energy");
  struc.energy() = e;
  return e;
}

static void force_impl(NNP& nnp, Structure& struc, bool no_vacuum, const char* where) {
  if (!nnp.ctx()) throw std::runtime_error(std::string(where) + ": no potential read");
  const Structure* p = &struc;
  Flat f;
  flatten(nnp, &p, 1, f);
  double e = 0.0;
  std::vector<double> F(3 * (size_t)std::max(struc.nAtoms(), 1));
  const int flags = NNPGPU_ENERGY | NNPGPU_FORCE | (no_vacuum ? NNPGPU_NO_VACUUM : 0) | (nnp.bf16() ? NNPGPU_BF16 : 0);
  check(nnp.ctx(), nnpgpu_compute(nnp.ctx(), 1, f.natoms.data(), f.posn.data(), f.species.data(), f.cell.data(), flags, &e, F.data(), nullptr),
        where);
  for (int i = 0; i < struc.nAtoms(); ++i)
    for (int x = 0; x < 3; ++x) struc.force(i)[x] = F[3 * (size_t)i + x];
  if (no_vacuum) struc.energy() = e;
}

void NNP::force(NNP& nnp, Structure& struc, const NeighborList&) { force_impl(nnp, struc, false, "NNP::force"); }

void NNP::compute(NNP& nnp, Structure& struc, const NeighborList&) { force_impl(nnp, struc, true, "NNP::compute"); }

void NNP::compute(NNP& nnp, std::vector<Structure>& strucs, bool force, bool no_vacuum) {
  if (!nnp.ctx_) throw std::runtime_error("NNP::compute: no potential read");
  if (strucs.empty()) return;
  std::vector<const Structure*> ptrs(strucs.size());
  for (size_t s = 0; s < strucs.size(); ++s) ptrs[s] = &strucs[s];
  Flat f;
  flatten(nnp, ptrs.data(), (int)ptrs.size(), f);
  std::vector<double> E(strucs.size()), F(force ? std::max<size_t>(f.posn.size(), 3) : 0);
  const int flags = NNPGPU_ENERGY | NNPGPU_BATCHED | (force ? NNPGPU_FORCE : 0) | (no_vacuum ? NNPGPU_NO_VACUUM : 0) |
                    (nnp.bf16_ ? NNPGPU_BF16 : 0);
  check(nnp.ctx(), nnpgpu_compute(nnp.ctx(), (int)strucs.size(), f.natoms.data(), f.posn.data(), f.species.data(), f.cell.data(), flags,
                                  E.data(), force ? F.data() : nullptr, nullptr),
        "NNP::compute (batched)");
  size_t a = 0;
  for (size_t s = 0; s < strucs.size(); ++s) {
    strucs[s].energy() = E[s];
    for (int i = 0; i < strucs[s].nAtoms(); ++i, ++a)
      if (force)
        for (int x = 0; x < 3; ++x) strucs[s].force(i)[x] = F[3 * a + x];
  }
}

// ------------------------------------------------------------------------------ NeighborList
void NeighborList::build(const Structure& struc, double rc) {
  std::shared_ptr<nnpgpu_ctx> c;
  {
    std::lock_guard<std::mutex> l(g_last_mu);
    c = g_last.lock();
  }
  if (!c) throw std::runtime_error("NeighborList::build: read a potential (NNP::read) first; it provides the GPU context");
  NNP tmp;
  tmp.ctx_ = c;
  build(tmp, struc, rc);
}

void NeighborList::build(const NNP& nnp, const Structure& struc, double rc) { build_atoms(nnp, struc, rc, {}, true); }

void NeighborList::build(const Structure& struc, double rc, int ii) {
  if (ii < 0 || ii >= struc.nAtoms()) throw std::invalid_argument("NeighborList::build: atom index out of range");
  std::vector<int> one(1, ii);
  build(struc, rc, one);
}

void NeighborList::build(const Structure& struc, double rc, const std::vector<int>& subset) {
  std::shared_ptr<nnpgpu_ctx> c;
  {
    std::lock_guard<std::mutex> l(g_last_mu);
    c = g_last.lock();
  }
  if (!c) throw std::runtime_error("NeighborList::build: read a potential (NNP::read) first; it provides the GPU context");
  for (int ii : subset)
    if (ii < 0 || ii >= struc.nAtoms()) throw std::invalid_argument("NeighborList::build: atom index out of range");
  NNP tmp;
  tmp.ctx_ = c;
  build_atoms(tmp, struc, rc, subset, false);
}

void NeighborList::build_atoms(const NNP& nnp, const Structure& struc, double rc, const std::vector<int>& subset, bool all) {
  if (!nnp.ctx()) throw std::runtime_error("NeighborList::build: no potential read");
  if (!(rc > 0)) throw std::invalid_argument("NeighborList::build: invalid cutoff");
  const int n = struc.nAtoms();
  std::vector<double> posn(3 * (size_t)std::max(n, 1));
  for (int i = 0; i < n; ++i)
    for (int x = 0; x < 3; ++x) posn[3 * (size_t)i + x] = struc.posn(i)[x];
  const std::array<double, 9>& R = struc.R();  // column-major, columns = lattice vectors
  double fro = 0.0;
  for (double v : R) fro += v * v;
  const bool periodic = fro > 0.0;
  std::vector<int> count(std::max(n, 1));
  int cap = 64;
  for (;;) {
    std::vector<int> index((size_t)std::max(n, 1) * cap), shift((size_t)std::max(n, 1) * cap * 3);
    std::vector<float> r((size_t)std::max(n, 1) * cap * 4);
    std::vector<unsigned char> mn((size_t)std::max(n, 1) * cap);
    const int code = nnpgpu_neighbors_rc(nnp.ctx(), rc, n, posn.data(), R.data(), cap, count.data(), index.data(), r.data(),
                                         mn.data(), shift.data());
    if (code == NNPGPU_ERR_CAPACITY && cap < 1024) {
      int need = cap;
      for (int i = 0; i < n; ++i) need = std::max(need, count[i]);
      cap = std::min(1024, (need + 31) / 32 * 32);
      continue;
    }
    check(nnp.ctx(), code, "NeighborList::build");
    rc_ = rc;
    if (all) neigh_.assign(n, {});
    else neigh_.resize(n);
    auto fill = [&](int i) {
      neigh_[i].resize(count[i]);
      for (int s = 0; s < count[i]; ++s) {
        const size_t g = (size_t)i * cap + s;
        Neighbor& nb = neigh_[i][s];
        const int j = index[g];
        const int T[3] = {shift[3 * g], shift[3 * g + 1], shift[3 * g + 2]};
        // r = posn(i) - posn(j) - R T in FP64 (the reference's rIJ - R_n, src/struc/neighbor.cpp:106-110)
        Vec3d v;
        for (int x = 0; x < 3; ++x) v[x] = struc.posn(i)[x] - struc.posn(j)[x] - (R[x] * T[0] + R[3 + x] * T[1] + R[6 + x] * T[2]);
        nb.r() = v;
        nb.dr() = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        nb.index() = (periodic && (int)struc.index().size() == n) ? struc.index(j) : j;
        nb.type() = ((int)struc.type().size() == n) ? struc.type(j) : -1;
        nb.min() = mn[g] != 0;
        nb.cell() = {T[0], T[1], T[2]};
      }
    };
    if (all)
      for (int i = 0; i < n; ++i) fill(i);
    else
      for (int i : subset) fill(i);
    return;
  }
}

// ------------------------------------------------------------------------------ readers
namespace VASP {
namespace POSCAR {
// VASP::POSCAR::read (src/format/vasp_struc.cpp:51-200): title, scale, three lattice vectors
// (one per line, each a column of R), species names, counts, a coordinate-mode line whose first
// character 'D' selects direct coordinates, then one position per atom.  Direct positions are
// mapped through the scaled lattice; Cartesian ones are multiplied by s_len only (the file's
// scale factor applies to the lattice alone, as in the reference).
void read(const char* file, Structure& struc, double s_len) {
  std::ifstream in(file ? file : "");
  if (!in) throw std::runtime_error(std::string("I/O Error: Could not open file: ") + (file ? file : "(null)"));
  std::string line;
  auto next = [&](const char* what) -> std::string {
    if (!std::getline(in, line)) throw std::runtime_error(std::string("POSCAR ") + file + ": missing " + what);
    return line;
  };
  next("title");
  double scale = 0.0;
  if (std::sscanf(next("scale").c_str(), "%lf", &scale) != 1) throw std::runtime_error(std::string("POSCAR ") + file + ": bad scale");
  double lv[9];
  for (int c = 0; c < 3; ++c)
    if (std::sscanf(next("lattice vector").c_str(), "%lf %lf %lf", &lv[3 * c], &lv[3 * c + 1], &lv[3 * c + 2]) != 3)
      throw std::runtime_error(std::string("POSCAR ") + file + ": bad lattice vector");
  for (double& v : lv) v *= s_len * scale;
  const std::vector<std::string> names = tokens(next("species names"));
  const std::vector<std::string> numbers = tokens(next("species counts"));
  if (names.size() != numbers.size()) throw std::runtime_error("Invalid number of species");
  if (names.empty()) throw std::runtime_error("Invalid number of species");
  std::vector<int> counts;
  int total = 0;
  for (const std::string& t : numbers) {
    counts.push_back(std::atoi(t.c_str()));
    total += counts.back();
  }
  const bool direct = !next("coordinate mode").empty() && line[0] == 'D';
  struc.clear();
  struc.init(lv);
  struc.resize(total);
  for (int n = 0; n < total; ++n) {
    double p[3];
    if (std::sscanf(next("position").c_str(), "%lf %lf %lf", &p[0], &p[1], &p[2]) != 3)
      throw std::runtime_error(std::string("POSCAR ") + file + ": bad position line " + std::to_string(n));
    for (int x = 0; x < 3; ++x)
      struc.posn(n)[x] = direct ? lv[x] * p[0] + lv[3 + x] * p[1] + lv[6 + x] * p[2] : p[x] * s_len;
  }
  int a = 0;
  for (size_t s = 0; s < names.size(); ++s)
    for (int m = 0; m < counts[s]; ++m, ++a) struc.name(a) = names[s];
}
}  // namespace POSCAR
}  // namespace VASP

namespace XYZ {
// XYZ::read (src/format/xyz_struc.cpp:38-130): atom count; a line "<tag> energy" or
// "<tag> energy a b c" (orthorhombic lattice lengths); then "name x y z" per atom.
void read(const char* file, Structure& struc, double s_len, double s_energy) {
  std::ifstream in(file ? file : "");
  if (!in) throw std::runtime_error(std::string("ERROR in XYZ::read: Could not open file: ") + (file ? file : "(null)"));
  std::string line;
  if (!std::getline(in, line)) throw std::runtime_error(std::string("XYZ ") + file + ": empty file");
  const int n = std::atoi(line.c_str());
  if (n <= 0) throw std::runtime_error("ERROR in XYZ::read: found zero atoms.");
  if (!std::getline(in, line)) throw std::runtime_error(std::string("XYZ ") + file + ": missing comment line");
  const std::vector<std::string> t = tokens(line);
  double energy = 0.0, lv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (t.size() == 2) {
    energy = std::atof(t[1].c_str());
  } else if (t.size() == 5) {
    energy = std::atof(t[1].c_str());
    lv[0] = std::atof(t[2].c_str()) * s_len;
    lv[4] = std::atof(t[3].c_str()) * s_len;
    lv[8] = std::atof(t[4].c_str()) * s_len;
  }
  struc.clear();
  struc.resize(n);
  for (int i = 0; i < n; ++i) {
    if (!std::getline(in, line)) throw std::runtime_error(std::string("XYZ ") + file + ": missing atom line " + std::to_string(i));
    char name[256];
    double p[3];
    if (std::sscanf(line.c_str(), "%255s %lf %lf %lf", name, &p[0], &p[1], &p[2]) != 4)
      throw std::runtime_error(std::string("XYZ ") + file + ": bad atom line " + std::to_string(i));
    struc.name(i) = name;
    for (int x = 0; x < 3; ++x) struc.posn(i)[x] = p[x] * s_len;
  }
  struc.init(lv);
  struc.energy() = s_energy * energy;
}
}  // namespace XYZ

// ------------------------------------------------------------------------------ parameters
bool boolean(const std::string& s) {
  return s == "T" || s == "t" || s == "TRUE" || s == "true" || s == "True" || s == "1";
}

ComputeParams read_compute_params(const char* file) {
  std::ifstream in(file ? file : "");
  if (!in) throw std::runtime_error("I/O Error: could not open parameter file.");
  ComputeParams p;
  std::string line;
  while (std::getline(in, line)) {
    const std::vector<std::string> t = tokens(line);
    if (t.empty()) continue;
    const std::string tag = upper(t[0]);
    const std::string val = t.size() > 1 ? t[1] : "";
    if (tag == "DATA") p.data.push_back(val);
    else if (tag == "NNPOT") p.nnpot = val;
    else if (tag == "FORMAT") p.format = upper(val);
    else if (tag == "UNITS") p.units = upper(val);
    else if (tag == "FORCE") p.force = boolean(val);
    else if (tag == "NORM") p.norm = boolean(val);
    else if (tag == "BF16") p.bf16 = boolean(val);
    else if (tag == "BATCH") p.batch_atoms = std::max(1LL, std::atoll(val.c_str()));
  }
  if (p.units != "METAL" && p.units != "AU") throw std::invalid_argument("Invalid unit system.");
  if (p.format != "POSCAR" && p.format != "XYZ") throw std::invalid_argument("Invalid file format.");
  if (p.data.empty()) throw std::invalid_argument("No data");
  return p;
}

std::vector<std::string> read_data_lists(const std::vector<std::string>& data) {
  std::vector<std::string> files;
  for (const std::string& d : data) {
    std::ifstream in(d);
    if (!in) throw std::runtime_error("I/O Error: Could not open data file: " + d);
    std::string line;
    while (std::getline(in, line)) {
      const size_t a = line.find_first_not_of(" \t\r\n");
      if (a == std::string::npos) continue;
      const size_t b = line.find_last_not_of(" \t\r\n");
      files.push_back(line.substr(a, b - a + 1));
    }
  }
  return files;
}

}  // namespace atomnn_gpu
