// potential.cpp - reader of AtomNN's potential text format and builder of the device tables.
#include "potential.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "../../include/nnpgpu.h"

namespace nnpgpu {

namespace {

const double kPi = 3.141592653589793;  // math::constant::PI (src/math/const.hpp:9)

std::vector<std::string> split_ws(const std::string& s) {  // string::WS tokens (src/str/string.hpp:16)
  std::vector<std::string> t;
  std::string cur;
  for (char ch : s) {
    if (ch == ' ' || ch == '\t' || ch == '\r' || ch == '\n') {
      if (!cur.empty()) t.push_back(cur), cur.clear();
    } else {
      cur.push_back(ch);
    }
  }
  if (!cur.empty()) t.push_back(cur);
  return t;
}

struct Lines {
  FILE* f;
  int lineno = 0;
  std::vector<std::string> next() {
    std::string s;
    int ch;
    bool any = false;
    while ((ch = std::fgetc(f)) != EOF) {
      any = true;
      if (ch == '\n') break;
      s.push_back((char)ch);
    }
    if (!any) throw PotError(NNPGPU_ERR_IO, "potential file: unexpected end of file after line " + std::to_string(lineno));
    ++lineno;
    return split_ws(s);
  }
};

const std::string& tok(const std::vector<std::string>& t, size_t i, const Lines& L) {
  if (i >= t.size()) throw PotError(NNPGPU_ERR_IO, "potential file: missing field on line " + std::to_string(L.lineno));
  return t[i];
}

int cut_of(const std::string& s) { return s == "STEP" ? CUT_STEP : s == "COS" ? CUT_COS : s == "TANH" ? CUT_TANH : 0; }
int norm_of(const std::string& s) { return s == "UNIT" ? 1 : s == "VOL" ? 2 : 0; }
double norm_value(int norm, double rc) {  // Basis::norm (src/nnp/basis.cpp:160-168)
  if (norm == 1) return 1.0;
  return 1.0 / (0.5 * 4.0 / 3.0 * (kPi * kPi - 6.0) / kPi * rc * rc * rc);
}

}  // namespace

HPot read_potential(const char* path) {
  FILE* f = std::fopen(path, "r");
  if (!f) throw PotError(NNPGPU_ERR_IO, std::string("could not open potential file \"") + path + "\"");
  HPot P;
  Lines L{f};
  try {
    L.next();  // "ann"
    auto t = L.next();
    P.ntypes = std::atoi(tok(t, 1, L).c_str());
    if (P.ntypes <= 0) throw PotError(NNPGPU_ERR_IO, "potential file: invalid number of types");
    P.types.resize(P.ntypes);
    for (int n = 0; n < P.ntypes; ++n) {  // Type::read (src/nnp/type.cpp:32-70)
      auto tt = L.next();
      for (size_t k = 0; k < tt.size(); ++k) {
        std::string tag = tt[k];
        if (!tag.empty() && tag[0] == '#') break;
        for (auto& c : tag) c = (char)std::toupper((unsigned char)c);
        const bool has = k + 1 < tt.size();
        if (tag == "NAME" && has) P.types[n].name = tt[++k];
        else if (tag == "MASS" && has) { P.types[n].mass = std::atof(tt[++k].c_str()); P.types[n].has_mass = true; }
        else if (tag == "ENERGY" && has) { P.types[n].energy = std::atof(tt[++k].c_str()); P.types[n].has_energy = true; }
        else if (has && (tag == "CHARGE" || tag == "CHI" || tag == "ETA" || tag == "JS" || tag == "C6" || tag == "RVDW" ||
                         tag == "RCOV"))
          P.types[n].other[tag] = std::atof(tt[++k].c_str());
      }
      P.index[P.types[n].name] = n;
    }
    t = L.next();
    P.rc = std::atof(tok(t, 1, L).c_str());
    if (!(P.rc > 0)) throw PotError(NNPGPU_ERR_IO, "potential file: invalid cutoff");
    const int nb = P.ntypes * (P.ntypes + 1) / 2;
    P.rad.assign(P.ntypes, std::vector<HBasisR>(P.ntypes));
    P.ang.assign(P.ntypes, std::vector<HBasisA>(nb));
    auto idx = [&](const std::string& s) {
      auto it = P.index.find(s);
      if (it == P.index.end()) throw PotError(NNPGPU_ERR_IO, "potential file: unknown type \"" + s + "\"");
      return it->second;
    };
    for (int i = 0; i < P.ntypes; ++i) {
      const int II = idx(tok(L.next(), 1, L));
      for (int j = 0; j < P.ntypes; ++j) {  // BasisR::read (src/nnp/basis_radial.cpp:123-144)
        const int JJ = idx(tok(L.next(), 1, L));
        auto h = L.next();
        HBasisR& b = P.rad[II][JJ];
        b.norm = norm_of(tok(h, 1, L));
        b.cut = cut_of(tok(h, 2, L));
        b.rc = std::atof(tok(h, 3, L).c_str());
        const std::string phi = tok(h, 4, L);
        b.phi = phi == "GAUSSIAN" ? RAD_GAUSSIAN : phi == "TANH" ? RAD_TANH : phi == "SOFTPLUS" ? RAD_SOFTPLUS
              : phi == "LOGCOSH" ? RAD_LOGCOSH : phi == "SWISH" ? RAD_SWISH : phi == "MISH" ? RAD_MISH : 0;
        if (b.phi == 0) throw PotError(NNPGPU_ERR_IO, "potential file: invalid radial function type " + phi);
        const int n = std::atoi(tok(h, 5, L).c_str());
        if (b.norm == 0) throw PotError(NNPGPU_ERR_IO, "potential file: invalid normalization scheme");
        if (!(b.rc > 0)) throw PotError(NNPGPU_ERR_IO, "potential file: invalid basis cutoff");
        for (int k = 0; k < n; ++k) {
          auto p = L.next();
          b.rs.push_back(std::atof(tok(p, 0, L).c_str()));
          b.eta.push_back(std::atof(tok(p, 1, L).c_str()));
        }
      }
      for (int j = 0; j < P.ntypes; ++j)
        for (int k = j; k < P.ntypes; ++k) {  // BasisA::read (src/nnp/basis_angular.cpp:113-138)
          auto tt = L.next();
          const int JJ = idx(tok(tt, 1, L)), KK = idx(tok(tt, 2, L));
          auto h = L.next();
          HBasisA& b = P.ang[II][lidx(JJ, KK)];
          b.norm = norm_of(tok(h, 1, L));
          b.cut = cut_of(tok(h, 2, L));
          b.rc = std::atof(tok(h, 3, L).c_str());
          const std::string phi = tok(h, 4, L);
          b.phi = phi == "GAUSS" ? ANG_GAUSS : phi == "IPOWP" ? ANG_IPOWP : phi == "IPOWS" ? ANG_IPOWS : phi == "SECHP" ? ANG_SECHP
                : phi == "SECHS" ? ANG_SECHS : 0;
          if (b.phi == 0) throw PotError(NNPGPU_ERR_IO, "potential file: invalid angular function type " + phi);
          const int n = std::atoi(tok(h, 5, L).c_str());
          b.alpha = std::atoi(tok(h, 6, L).c_str());
          if (b.norm == 0) throw PotError(NNPGPU_ERR_IO, "potential file: invalid normalization scheme");
          if (!(b.rc > 0)) throw PotError(NNPGPU_ERR_IO, "potential file: invalid basis cutoff");
          for (int q = 0; q < n; ++q) {
            auto p = L.next();
            b.eta.push_back(std::atof(tok(p, 0, L).c_str()));
            b.zeta.push_back(std::atof(tok(p, 1, L).c_str()));
            b.lam.push_back(std::atoi(tok(p, 2, L).c_str()));
          }
        }
    }
    // input layout (NNH::init_input, src/nnp/nnh.cpp:95-121)
    P.nin.assign(P.ntypes, 0);
    P.ninR.assign(P.ntypes, 0);
    P.offR.assign(P.ntypes, std::vector<int>(P.ntypes, 0));
    P.offA.assign(P.ntypes, std::vector<int>(nb, 0));
    for (int I = 0; I < P.ntypes; ++I) {
      int r = 0;
      for (int J = 0; J < P.ntypes; ++J) { P.offR[I][J] = r; r += (int)P.rad[I][J].rs.size(); }
      int a = 0;
      for (int b = 0; b < nb; ++b) { P.offA[I][b] = a; a += (int)P.ang[I][b].eta.size(); }
      P.ninR[I] = r;
      P.nin[I] = r + a;
    }
    // networks (ANN::read, src/ml/nn.cpp:1349-1425)
    P.nets.resize(P.ntypes);
    for (int n = 0; n < P.ntypes; ++n) {
      const int II = idx(tok(L.next(), 1, L));
      HNet& net = P.nets[II];
      auto cfg = L.next();
      std::vector<int> nodes;
      for (size_t k = 1; k < cfg.size(); ++k) nodes.push_back(std::atoi(cfg[k].c_str()));
      if (nodes.size() < 2) throw PotError(NNPGPU_ERR_IO, "potential file: invalid network configuration");
      net.nin = nodes[0];
      net.nodes.assign(nodes.begin() + 1, nodes.end());
      for (int x : nodes)
        if (x <= 0) throw PotError(NNPGPU_ERR_IO, "potential file: invalid layer size");
      const std::string neuron = tok(L.next(), 1, L);
      net.neuron = neuron;
      net.act = neuron == "TANH" ? ACT_TANH : neuron == "LINEAR" ? ACT_LINEAR : neuron == "SIGMOID" ? ACT_SIGMOID : -1;
      if (net.act < 0) {
        static const char* known[] = {"ISRU", "ARCTAN", "SOFTSIGN", "RELU", "SOFTPLUS", "ELU", "GELU", "SWISH", "MISH",
                                      "TANHRE", "LOGCOSH", "IQUAD", "IFABS", "SINSIG"};
        bool k = false;
        for (const char* s : known) k = k || neuron == s;
        if (!k) throw PotError(NNPGPU_ERR_IO, "potential file: invalid neuron " + neuron);
        net.act = 0;  // valid in the reference, not implemented here
      }
      const int nout = net.nodes.back();
      auto vec = [&](std::vector<double>& v, int cnt) {
        auto p = L.next();
        v.resize(cnt);
        for (int k = 0; k < cnt; ++k) v[k] = std::atof(tok(p, k + 1, L).c_str());
      };
      vec(net.inpw, net.nin);
      vec(net.outw, nout);
      vec(net.inpb, net.nin);
      vec(net.outb, nout);
      const int Ln = (int)net.nodes.size();
      net.b.resize(Ln);
      net.w.resize(Ln);
      for (int l = 0; l < Ln; ++l) vec(net.b[l], net.nodes[l]);
      for (int l = 0; l < Ln; ++l) vec(net.w[l], net.nodes[l] * (l == 0 ? net.nin : net.nodes[l - 1]));
      if (net.nin != P.nin[II]) throw PotError(NNPGPU_ERR_IO, "potential file: network input size does not match the basis");
    }
  } catch (...) {
    std::fclose(f);
    throw;
  }
  std::fclose(f);
  return P;
}

void build_tables(const HPot& pot, PotParams& P, int& ne_max, int& nz_max) {
  auto unsup = [](const std::string& m) { throw PotError(NNPGPU_ERR_UNSUPPORTED, m); };
  P = PotParams();
  if (pot.ntypes > NT_MAX) unsup("more than " + std::to_string(NT_MAX) + " atom types");
  P.ntypes = pot.ntypes;
  P.rc = (float)pot.rc;
  ne_max = 1;
  nz_max = 1;
  P.mstride = 0;
  for (int I = 0; I < pot.ntypes; ++I) {
    int moff = 0;  // moment floats of this centre type so far
    if (pot.nin[I] > NIN_MAX) unsup("more than " + std::to_string(NIN_MAX) + " network inputs");
    P.nin[I] = pot.nin[I];
    for (int J = 0; J < pot.ntypes; ++J) {
      const HBasisR& b = pot.rad[I][J];
      RadialP& r = P.rad[I][J];

      if ((int)b.rs.size() > NR_MAX) unsup("more than " + std::to_string(NR_MAX) + " radial functions per pair");
      if (b.cut == 0) unsup("unknown cutoff function");
      r.n = (int)b.rs.size();
      r.off = pot.offR[I][J];
      r.cut = b.cut;
      r.phi = b.phi;
      r.rc = (float)b.rc;
      r.pirc = (float)(kPi / b.rc);
      r.rci = (float)(1.0 / b.rc);
      r.norm = (float)norm_value(b.norm, b.rc);
      for (int k = 0; k < r.n; ++k) { r.rs[k] = (float)b.rs[k]; r.eta[k] = (float)b.eta[k]; }
    }
    for (int q = 0; q < pot.ntypes * (pot.ntypes + 1) / 2; ++q) {
      const HBasisA& b = pot.ang[I][q];
      AngP& a = P.ang[I][q];
      const int n = (int)b.eta.size();
      if (n == 0) continue;
      if (b.phi < ANG_GAUSS || b.phi > ANG_SECHS) unsup("unknown angular function");
      if (n > NA_MAX) unsup("more than " + std::to_string(NA_MAX) + " angular functions per block");
      if (b.cut == 0) unsup("unknown cutoff function");
      if (b.alpha < 1 || b.alpha > 8) unsup("angular power alpha outside 1..8");
      a.n = n;
      a.off = pot.ninR[I] + pot.offA[I][q];
      a.cut = b.cut;
      a.phi = b.phi;
      if (b.phi != ANG_GAUSS) P.gen = 1;
      a.alpha = b.alpha;
      a.rc = (float)b.rc;
      a.pirc = (float)(kPi / b.rc);
      a.rci = (float)(1.0 / b.rc);
      a.norm = (float)norm_value(b.norm, b.rc);
      std::vector<double> ie;   // distinct 1/eta^alpha (BasisA::init, basis_angular.cpp:168-173)
      std::vector<int> lams;
      for (int f = 0; f < n; ++f) {
        double v = 1.0;
        for (int k = 0; k < b.alpha; ++k) v *= 1.0 / b.eta[f];
        if (std::find(ie.begin(), ie.end(), v) == ie.end()) ie.push_back(v);
        if (std::find(lams.begin(), lams.end(), b.lam[f]) == lams.end()) lams.push_back(b.lam[f]);
      }
      // blocks whose functions leave the (width) x (lambda) x (zeta = 2^m) grid - real zeta, more
      // than NE_MAX widths or NL lambdas - take the per-function path (a.fn) of the GEN kernels
      bool fn = (int)ie.size() > NE_MAX || (int)lams.size() > NL;
      for (int f = 0; f < n; ++f) {
        bool pow2 = false;
        for (int k = 0; k < NZ_MAX; ++k) pow2 = pow2 || b.zeta[f] == (double)(1 << k);
        if (!pow2) fn = true;
        if (!(b.zeta[f] >= 1.0) || !std::isfinite(b.zeta[f])) unsup("angular zeta below 1 or not finite");
      }
      if (fn) {
        a.fn = 1;
        a.ne = 1;
        a.nl = 1;
        a.nz = 1;
        a.mom = 0;
        P.gen = 1;
        continue;
      }
      a.ne = (int)ie.size();
      a.nl = (int)lams.size();
      for (int e = 0; e < a.ne; ++e) a.ietap[e] = (float)ie[e];
      for (int l = 0; l < NL; ++l) a.lam[l] = l < a.nl ? (float)lams[l] : 0.f;
      int nz = 1;
      for (int f = 0; f < n; ++f) {
        int m = -1;
        for (int k = 0; k < NZ_MAX; ++k)
          if (b.zeta[f] == (double)(1 << k)) m = k;
        if (m < 0) unsup("zeta values other than powers of two up to " + std::to_string(1 << (NZ_MAX - 1)));
        nz = std::max(nz, m + 1);
        double v = 1.0;
        for (int k = 0; k < b.alpha; ++k) v *= 1.0 / b.eta[f];
        const int e = (int)(std::find(ie.begin(), ie.end(), v) - ie.begin());
        const int l = (int)(std::find(lams.begin(), lams.end(), b.lam[f]) - lams.begin());
        a.gidx[f] = (signed char)((e * NL + l) * NZ_MAX + m);
      }
      a.nz = nz;
      // zeta <= 4 with |lambda| <= 1: ((1 + lambda cos)/2)^zeta is a polynomial of degree <= 4
      // in cos with a non-negative base, which the moment-tensor path evaluates when the radial
      // factor is a product h(r_ij) h(r_ik)
      bool lam_ok = true;
      for (int l = 0; l < a.nl; ++l) lam_ok = lam_ok && std::fabs((double)lams[l]) <= 1.0;
      // a GAUSS block whose functions have zeta <= MOM_N or the block's largest zeta (above
      // MOM_N) splits: the low ones take the moment path, the top level the triplet path
      bool split = b.phi == ANG_GAUSS && lam_ok && (1 << (nz - 1)) > MOM_N;
      bool any_low = false;
      for (int f = 0; split && f < n; ++f) {
        const int m = a.gidx[f] % NZ_MAX;
        if ((1 << m) <= MOM_N) any_low = true;
        else if (m != nz - 1) split = false;
      }
      split = split && any_low;
      if (((1 << (nz - 1)) <= MOM_N && lam_ok && !ang_sum_family(b.phi)) || split) {
        int J = 0, K = 0;
        for (int x = 0; x < pot.ntypes; ++x)
          for (int y = x; y < pot.ntypes; ++y)
            if (lidx(x, y) == q) { J = x; K = y; }
        a.mom = 1;
        a.top = split ? 1 : 0;
        a.moff = moff;
        moff += (J == K ? 1 : 2) * a.ne * MOM_C;
      }
      if (!a.mom || a.top) {
        nz_max = std::max(nz_max, nz);  // the triplet kernels' zeta chain covers triplet blocks only
        if (b.phi == ANG_IPOWP || b.phi == ANG_SECHP) P.kx = 1;
      }
      ne_max = std::max(ne_max, a.ne);
    }
    // moment blocks that share one pair weight (widths, alpha, cutoff, radius, family) and at
    // most two neighbour species: the kernels build each species' moments once per centre and
    // contract each neighbour once against the sum of its blocks' tables
    {
      std::vector<int> mq;
      for (int q = 0; q < pot.ntypes * (pot.ntypes + 1) / 2; ++q)
        if (P.ang[I][q].n > 0 && P.ang[I][q].mom) mq.push_back(q);
      bool ok = mq.size() >= 2;
      std::vector<int> sp;
      int rep = ok ? mq[0] : 0;  // the block with the most widths
      for (size_t t = 0; ok && t < mq.size(); ++t)
        if (P.ang[I][mq[t]].ne > P.ang[I][rep].ne) rep = mq[t];
      for (size_t t = 0; ok && t < mq.size(); ++t) {
        const AngP& a = P.ang[I][mq[t]];
        const AngP& r = P.ang[I][rep];
        ok = a.alpha == r.alpha && a.cut == r.cut && a.rc == r.rc && a.phi == r.phi;
        for (int e = 0; ok && e < a.ne; ++e) ok = std::find(r.ietap, r.ietap + r.ne, a.ietap[e]) != r.ietap + r.ne;
        for (int x = 0; x < pot.ntypes; ++x)
          for (int y = x; y < pot.ntypes; ++y)
            if (lidx(x, y) == mq[t]) {
              if (std::find(sp.begin(), sp.end(), x) == sp.end()) sp.push_back(x);
              if (std::find(sp.begin(), sp.end(), y) == sp.end()) sp.push_back(y);
            }
      }
      ok = ok && sp.size() <= 2 && mq.size() <= 3;
      if (ok) {
        std::sort(sp.begin(), sp.end());
        P.msh[I] = 1;
        P.mns[I] = (int)sp.size();
        P.mrep[I] = rep;
        for (int t = 0; t < 2; ++t) P.msp[I][t] = t < (int)sp.size() ? sp[t] : -1;
        moff = P.mns[I] * P.ang[I][rep].ne * MOM_C;  // the shared moments replace the per-block ones
      }
    }
    P.mstride = std::max(P.mstride, (moff + 3) / 4 * 4);
    // one cutoff function and radius for every basis of this centre type: the kernels then
    // evaluate it once per neighbour
    {
      int cut = 0;
      double rcv = 0.0;
      bool same = true, any = false;
      auto see = [&](int c, double r) {
        if (!any) { cut = c; rcv = r; any = true; }
        else if (c != cut || r != rcv) same = false;
      };
      for (int J = 0; J < pot.ntypes; ++J)
        if (!pot.rad[I][J].rs.empty()) see(pot.rad[I][J].cut, pot.rad[I][J].rc);
      for (int q = 0; q < pot.ntypes * (pot.ntypes + 1) / 2; ++q)
        if (!pot.ang[I][q].eta.empty()) see(pot.ang[I][q].cut, pot.ang[I][q].rc);
      P.ccut[I] = (same && any) ? cut : 0;
      P.crc[I] = (float)rcv;
      P.cpirc[I] = any ? (float)(kPi / rcv) : 0.f;
      P.crci[I] = any ? (float)(1.0 / rcv) : 0.f;
    }
    const HNet& net = pot.nets[I];
    if (net.act <= 0) unsup("network activation not implemented on the GPU");
    if ((int)net.nodes.size() < 2 || (int)net.nodes.size() > NLAYER_MAX) unsup("networks need 1 to 3 hidden layers");
    if (net.nodes.back() != 1) unsup("networks with more than one output");
    for (int x : net.nodes)
      if (x > HID_MAX) unsup("layers wider than " + std::to_string(HID_MAX));
  }
}

std::vector<float> build_ang_tables(const HPot& pot, PotParams& P) {
  std::vector<float> tab;
  for (int I = 0; I < pot.ntypes; ++I)
    for (int q = 0; q < pot.ntypes * (pot.ntypes + 1) / 2; ++q) {
      AngP& a = P.ang[I][q];
      if (a.n == 0) continue;
      while (tab.size() % 4) tab.push_back(0.f);
      a.tab = (int)tab.size();
      const HBasisA& b = pot.ang[I][q];
      if (a.fn) {
        // per function: 1/eta^alpha (BasisA::init, basis_angular.cpp:168-173), lambda, zeta, 0
        for (int f = 0; f < a.n; ++f) {
          double ie = 1.0;
          for (int k = 0; k < b.alpha; ++k) ie *= 1.0 / b.eta[f];
          tab.push_back((float)ie);
          tab.push_back((float)b.lam[f]);
          tab.push_back((float)b.zeta[f]);
          tab.push_back(0.f);
        }
        continue;
      }
      for (int f = 0; f < a.n; ++f) tab.push_back((float)a.gidx[f]);
      if (!a.mom) continue;
      // columns follow the widths of the block whose moments this block reads: its own, or
      // those of the centre type's representative block when the moments are shared
      const AngP& L = P.msh[I] ? P.ang[I][P.mrep[I]] : a;
      const int w = L.ne * (MOM_N + 1);
      const double norm = norm_value(b.norm, b.rc);
      for (int f = 0; f < a.n; ++f) {
        const int cell = a.gidx[f];
        const int m = cell % NZ_MAX, zeta = 1 << m;
        const int e = (int)(std::find(L.ietap, L.ietap + L.ne, a.ietap[cell / (NL * NZ_MAX)]) - L.ietap);
        const double lam = a.lam[(cell / NZ_MAX) % NL];
        // ((1 + lam c)/2)^zeta = sum_k binom(zeta, k) / 2^zeta lam^k c^k; functions of a split
        // block's top level (zeta > MOM_N) are the triplet path's: zero rows
        for (int col = 0; col < w; ++col) {
          const int ce = col / (MOM_N + 1), k = col % (MOM_N + 1);
          double v = 0.0;
          if (ce == e && k <= zeta && zeta <= MOM_N) {
            double binom = 1.0;
            for (int j = 0; j < k; ++j) binom = binom * (zeta - j) / (j + 1);
            v = norm * binom * std::pow(lam, k) / (double)(1 << zeta);
          }
          tab.push_back((float)v);
        }
      }
    }
  return tab;
}

void write_potential(const HPot& P, const char* path) {
  FILE* f = std::fopen(path, "w");
  if (!f) throw PotError(NNPGPU_ERR_IO, std::string("could not open \"") + path + "\" for writing");
  static const char* cut_names[] = {"UNKNOWN", "STEP", "COS", "TANH"};
  static const char* norm_names[] = {"UNKNOWN", "UNIT", "VOL"};
  static const char* rad_names[] = {"UNKNOWN", "GAUSSIAN", "TANH", "SOFTPLUS", "LOGCOSH", "SWISH", "MISH"};
  static const char* ang_names[] = {"UNKNOWN", "GAUSS", "IPOWP", "IPOWS", "SECHP", "SECHS"};
  auto name = [](const char* const* names, int n, int v) { return (v >= 0 && v < n) ? names[v] : names[0]; };
  std::fprintf(f, "ann\n");
  std::fprintf(f, "ntypes %i\n", P.ntypes);
  for (const HType& t : P.types) {  // Type::write (src/nnp/type.cpp:125-138): flagged properties in this order
    std::fprintf(f, "name %s ", t.name.c_str());
    if (t.has_mass) std::fprintf(f, "mass %f ", t.mass);
    if (t.has_energy) std::fprintf(f, "energy %f ", t.energy);
    for (const char* key : {"CHARGE", "CHI", "ETA", "JS", "C6", "RVDW", "RCOV"}) {
      auto it = t.other.find(key);
      if (it == t.other.end()) continue;
      std::string low(key);
      for (char& ch : low) ch = (char)std::tolower((unsigned char)ch);
      std::fprintf(f, "%s %f ", low.c_str(), it->second);
    }
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "rc %f\n", P.rc);
  for (int i = 0; i < P.ntypes; ++i) {
    std::fprintf(f, "basis %s\n", P.types[i].name.c_str());
    for (int j = 0; j < P.ntypes; ++j) {  // BasisR::write (src/nnp/basis_radial.cpp:107-116)
      const HBasisR& b = P.rad[i][j];
      std::fprintf(f, "basis_radial %s\n", P.types[j].name.c_str());
      std::fprintf(f, "BasisR %s %s %f %s %i\n", name(norm_names, 3, b.norm), name(cut_names, 4, b.cut), b.rc, name(rad_names, 7, b.phi),
                   (int)b.rs.size());
      for (size_t k = 0; k < b.rs.size(); ++k) std::fprintf(f, "\t%f %f\n", b.rs[k], b.eta[k]);
    }
    for (int j = 0; j < P.ntypes; ++j)
      for (int k = j; k < P.ntypes; ++k) {  // BasisA::write (src/nnp/basis_angular.cpp:97-106)
        const HBasisA& b = P.ang[i][lidx(j, k)];
        std::fprintf(f, "basis_angular %s %s\n", P.types[j].name.c_str(), P.types[k].name.c_str());
        std::fprintf(f, "BasisA %s %s %f %s %i %i\n", name(norm_names, 3, b.norm), name(cut_names, 4, b.cut), b.rc, name(ang_names, 6, b.phi),
                     (int)b.eta.size(), b.alpha);
        for (size_t q = 0; q < b.eta.size(); ++q) std::fprintf(f, "\t%f %f %i\n", b.eta[q], b.zeta[q], b.lam[q]);
      }
  }
  for (int n = 0; n < P.ntypes; ++n) {  // ANN::write (src/ml/nn.cpp:1284-1323)
    const HNet& net = P.nets[n];
    std::fprintf(f, "nn %s\n", P.types[n].name.c_str());
    std::fprintf(f, "nn %i ", net.nin);
    for (int x : net.nodes) std::fprintf(f, "%i ", x);
    std::fprintf(f, "\n");
    std::fprintf(f, "neuron %s\n", net.neuron.c_str());
    auto row = [&](const char* tag, const std::vector<double>& v) {
      std::fprintf(f, "%s ", tag);
      for (double x : v) std::fprintf(f, "%.15f ", x);
      std::fprintf(f, "\n");
    };
    row("inpw", net.inpw);
    row("outw", net.outw);
    row("inpb", net.inpb);
    row("outb", net.outb);
    for (size_t l = 0; l < net.b.size(); ++l) row(("bias[" + std::to_string(l + 1) + "]").c_str(), net.b[l]);
    for (size_t l = 0; l < net.w.size(); ++l)
      row(("weight[" + std::to_string(l) + "," + std::to_string(l + 1) + "]").c_str(), net.w[l]);
  }
  const bool ok = std::ferror(f) == 0;
  if (std::fclose(f) != 0 || !ok) throw PotError(NNPGPU_ERR_IO, std::string("write error on \"") + path + "\"");
}

}  // namespace nnpgpu
