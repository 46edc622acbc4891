// nnp_oracle.cpp - FP64 CPU oracle of AtomNN's NNP energy/force path.
//
// TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels, never part of the product.
// Parity status: unpinned against the reference binary (Eigen 3.4 and MPI are absent, so the
// reference cannot be compiled; its tests hold no golden vectors).  Pinned by the reference's
// own test properties instead: see nnp_oracle.h.
//
// Each function below restates one reference routine in plain C++17 (no Eigen) and names the
// reference file:line it follows.  Matrix-vector products are written as explicit sums in
// index order; the reference evaluates them through Eigen, so agreement is to rounding, not
// to the bit, except where noted.
//
// Build: plain g++ with -ffp-contract=off so that the x86 and Arm builds give the same bits.
#include "nnp_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

typedef std::array<double, 3> V3;
static const double PI = 3.141592653589793;  // math::constant::PI, src/math/const.hpp:9
static const double ZERO = 1e-6;             // math::constant::ZERO, src/math/const.hpp:8

static inline double dot(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline double sqn(const V3& a) { return dot(a, a); }
static inline double nrm(const V3& a) { return std::sqrt(sqn(a)); }
static inline V3 cross(const V3& a, const V3& b) {
  return V3{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}

// ---------------------------------------------------------------- math helpers
// math::special::powint, src/math/special.cpp:111-120
static double powint(double x, int n) {
  if (n == 0) return 1.0;
  if (x == 0.0) return 0.0;
  int nn = (n > 0) ? n : -n;
  double ww = x, yy = 1.0;
  for (; nn != 0; nn >>= 1, ww *= ww)
    if (nn & 1) yy *= ww;
  return (n > 0) ? yy : 1.0 / yy;
}
// math::special::sech, src/math/special.cpp:71-79
static double sech(double x) {
  if (x >= 0) { const double e = std::exp(-x); return 2.0 * e / (1.0 + e * e); }
  const double e = std::exp(x);
  return 2.0 * e / (e * e + 1.0);
}
// math::special::logp1 (truncated 2*atanh series, not log1p), src/math/special.cpp:131-135
static double logp1(double x) {
  const double y = x / (x + 2.0);
  const double y2 = y * y;
  return 2.0 * y * (1.0 + y2 * (1.0 / 3.0 + y2 * (1.0 / 5.0 + y2 * (1.0 / 7.0 + y2 * 1.0 / 9.0))));
}
// math::special::mod (real), src/math/special.hpp:43-46
static inline double fmod2(double n, double z) { return std::fmod(std::fmod(n, z) + z, z); }
static inline double modlim(double n, double lo, double hi) { return fmod2(n - lo, hi - lo) + lo; }

// ---------------------------------------------------------------- basis
enum CutName { CUT_UNKNOWN = 0, CUT_STEP, CUT_COS, CUT_TANH };      // src/nnp/cutoff.hpp:56-61
enum CutNorm { NORM_UNKNOWN = 0, NORM_UNIT, NORM_VOL };             // src/nnp/cutoff.hpp:29-33
enum PhiR { PR_UNKNOWN = 0, PR_GAUSSIAN, PR_TANH, PR_SOFTPLUS, PR_LOGCOSH, PR_SWISH, PR_MISH };  // basis_radial.hpp:25-33
enum PhiA { PA_UNKNOWN = 0, PA_GAUSS, PA_IPOWP, PA_IPOWS, PA_SECHP, PA_SECHS };                 // basis_angular.hpp:25-32

struct Basis {
  int cutname = CUT_UNKNOWN, cutnorm = NORM_UNKNOWN, size = 0;
  double rc = 0, rci = 0, pirci = 0, norm = 0;
  // Basis::Basis(rc,...), src/nnp/basis.cpp:33-46 ; Basis::norm, :160-168
  void init(double rc_, int name, int nrm_) {
    if (rc_ <= 0) throw std::invalid_argument("Basis: invalid cutoff radius");
    rc = rc_; rci = 1.0 / rc; pirci = PI / rc; cutname = name; cutnorm = nrm_;
    if (nrm_ == NORM_UNIT) norm = 1.0;
    else if (nrm_ == NORM_VOL) norm = 1.0 / (0.5 * 4.0 / 3.0 * (PI * PI - 6.0) / PI * rc * rc * rc);
    else throw std::invalid_argument("Basis::norm: invalid normalization scheme");
  }
  // Basis::cut_func, src/nnp/basis.cpp:80-98
  double cut_func(double dr) const {
    switch (cutname) {
      case CUT_STEP: return (dr > rc) ? 0.0 : 1.0;
      case CUT_COS: return (dr > rc) ? 0 : 0.5 * (std::cos(dr * pirci) + 1.0);
      case CUT_TANH: { const double f = (dr > rc) ? 0 : std::tanh(1.0 - dr * rci); return f * f * f; }
      default: throw std::invalid_argument("Basis::cut_func: invalid cutoff type");
    }
  }
  // Basis::cut_grad, src/nnp/basis.cpp:100-120
  double cut_grad(double dr) const {
    switch (cutname) {
      case CUT_STEP: return 0.0;
      case CUT_COS: return (dr > rc) ? 0 : -0.5 * pirci * std::sin(dr * pirci);
      case CUT_TANH:
        if (dr < rc) { const double f = std::tanh(1.0 - dr * rci); return -3.0 * f * f * (1.0 - f * f) * rci; }
        return 0;
      default: throw std::invalid_argument("Basis::cut_grad: invalid cutoff type");
    }
  }
};

struct BasisR : Basis {
  int phi = PR_UNKNOWN;
  std::vector<double> rs, eta;
  // BasisR::symm(double), src/nnp/basis_radial.cpp:302-364 ; adds into out[0..size)
  void symm_add(double dr, double* out) const {
    const double cut = cut_func(dr) * norm;
    for (int i = 0; i < size; ++i) {
      const double arg = -eta[i] * (dr - rs[i]);
      double v = 0;
      switch (phi) {
        case PR_GAUSSIAN: v = std::exp(-eta[i] * (dr - rs[i]) * (dr - rs[i])) * cut; break;
        case PR_TANH: v = 0.5 * (std::tanh(-eta[i] * (dr - rs[i])) + 1.0) * cut; break;
        case PR_SOFTPLUS:
          v = (arg > 0.0) ? (arg + logp1(std::exp(-arg))) * cut : logp1(std::exp(arg)) * cut; break;
        case PR_LOGCOSH:
          v = (arg > 0.0) ? (arg + 0.5 * logp1(std::exp(-2.0 * arg))) * cut : 0.5 * logp1(std::exp(2.0 * arg)) * cut;
          break;
        case PR_SWISH:
          if (arg > 0.0) { const double e = std::exp(-arg); v = arg / (1.0 + e) * cut; }
          else if (arg < 0.0) { const double e = std::exp(arg); v = arg * e / (1.0 + e) * cut; }
          break;
        case PR_MISH:
          if (arg > 0.0) { const double e = std::exp(-arg); v = arg * (2.0 * e + 1.0) / (2.0 * e * (e + 1.0) + 1.0) * cut; }
          else if (arg < 0.0) { const double e = std::exp(arg); v = arg * e * (e + 2.0) / (e * (e + 2.0) + 2.0) * cut; }
          break;
        default: throw std::invalid_argument("BasisR::symm: invalid symmetry function");
      }
      out[i] += v;
    }
  }
  // BasisR::force(double,const double*), src/nnp/basis_radial.cpp:371-444
  double force(double dr, const double* dEdG) const {
    double amp = 0;
    const double cut = cut_func(dr), gcut = cut_grad(dr);
    for (int i = 0; i < size; ++i) {
      const double arg = -eta[i] * (dr - rs[i]);
      switch (phi) {
        case PR_GAUSSIAN:
          amp -= dEdG[i] * std::exp(-eta[i] * (dr - rs[i]) * (dr - rs[i])) * (-2.0 * eta[i] * (dr - rs[i]) * cut + gcut);
          break;
        case PR_TANH: {
          const double t = std::tanh(-eta[i] * (dr - rs[i]));
          amp -= dEdG[i] * 0.5 * (-eta[i] * (1.0 - t * t) * cut + (1.0 + t) * gcut);
        } break;
        case PR_SOFTPLUS:
          if (arg > 0.0) { const double e = std::exp(-arg); amp -= dEdG[i] * (-eta[i] * 1.0 / (1.0 + e) * cut + (arg + logp1(e)) * gcut); }
          else { const double e = std::exp(arg); amp -= dEdG[i] * (-eta[i] * e / (1.0 + e) * cut + logp1(e) * gcut); }
          break;
        case PR_LOGCOSH:
          if (arg > 0.0) { const double e = std::exp(-2.0 * arg); amp -= dEdG[i] * (-eta[i] / (1.0 + e) * cut + (arg + 0.5 * logp1(e)) * gcut); }
          else { const double e = std::exp(2.0 * arg); amp -= dEdG[i] * (-eta[i] * e / (1.0 + e) * cut + 0.5 * logp1(e) * gcut); }
          break;
        case PR_SWISH:
          if (arg > 0) {
            const double e = std::exp(-arg), den = 1.0 / (1.0 + e);
            amp -= dEdG[i] * (-eta[i] * (1.0 + e * (1.0 + arg)) * den * cut + arg * gcut) * den;
          } else {
            const double e = std::exp(arg), den = 1.0 / (1.0 + e);
            amp -= dEdG[i] * (-eta[i] * (1.0 + arg + e) * den * cut + arg * gcut) * e * den;
          }
          break;
        case PR_MISH:
          if (arg > 0.0) {
            const double e = std::exp(-arg), den = 1.0 / (2.0 * e * (e + 1.0) + 1.0);
            amp -= dEdG[i] * (-eta[i] * (1.0 + e * (4.0 + e * (4.0 * arg + 6.0 + e * 4.0 * (arg + 1.0)))) * den * cut +
                              arg * (2.0 * e + 1.0) * gcut) * den;
          } else {
            const double e = std::exp(arg), den = 1.0 / (e * (e + 2.0) + 2.0);
            amp -= dEdG[i] * (-eta[i] * (e * (e * (e + 4.0) + 4.0 * arg + 6.0) + 4.0 * (arg + 1.0)) * den * cut +
                              arg * (e + 2.0) * gcut) * den * e;
          }
          break;
        default: throw std::invalid_argument("BasisR::force: invalid symmetry function");
      }
    }
    return amp * norm;
  }
  // d G_m / d r for every function m: the term BasisR::force contracts with dE/dG (force
  // returns -sum_m dEdG_m dG_m/dr); evaluated through force with a unit dE/dG per function.
  void dval(double dr, double* out) const {
    std::vector<double> unit(size, 0.0);
    for (int m = 0; m < size; ++m) {
      unit[m] = 1.0;
      out[m] = -force(dr, unit.data());
      unit[m] = 0.0;
    }
  }
};

struct BasisA : Basis {
  int phi = PA_UNKNOWN, alpha = 0;
  std::vector<double> eta, zeta, ietap;
  std::vector<int> lambda;
  // BasisA::init, src/nnp/basis_angular.cpp:168-173
  void init_ietap() {
    ietap.resize(size);
    for (int i = 0; i < size; ++i) ietap[i] = powint(1.0 / eta[i], alpha);
  }
  // BasisA::symm(double,const double*), src/nnp/basis_angular.cpp:406-446 ; adds into out
  void symm_add(double cs, const double d[3], double* out) const {
    const double c0 = cut_func(d[0]), c1 = cut_func(d[1]);
    const double cprod = c0 * c1 * norm;
    const double rijp = powint(d[0], alpha), rikp = powint(d[1], alpha);
    for (int i = 0; i < size; ++i) {
      const double ang = std::pow(std::fabs(0.5 * (1.0 + lambda[i] * cs)), zeta[i]) * cprod;
      double v = 0;
      switch (phi) {
        case PA_GAUSS: v = ang * std::exp(-ietap[i] * (rijp + rikp)); break;
        case PA_IPOWP: v = ang * 1.0 / ((1.0 + ietap[i] * rijp) * (1.0 + ietap[i] * rikp)); break;
        case PA_IPOWS: v = ang * 1.0 / (1.0 + ietap[i] * (rijp + rikp)); break;
        case PA_SECHP: v = ang * sech(ietap[i] * rijp) * sech(ietap[i] * rikp); break;
        case PA_SECHS: v = ang * sech(ietap[i] * (rijp + rikp)); break;
        default: throw std::invalid_argument("BasisA::symm: invalid symmetry function");
      }
      out[i] += v;
    }
  }
  // BasisA::force(double&,double*,double,const double[3],const double*), src/nnp/basis_angular.cpp:456-640
  void force(double& phi_o, double* eta_o, double cs, const double d[3], const double* dEdG) const {
    const double c[2] = {cut_func(d[0]), cut_func(d[1])};
    const double g[2] = {cut_grad(d[0]), cut_grad(d[1])};
    phi_o = 0; eta_o[0] = 0; eta_o[1] = 0; eta_o[2] = 0;
    const double cprod = c[0] * c[1];
    const double rijp = powint(d[0], alpha), rikp = powint(d[1], alpha);
    const double dij = alpha * rijp / d[0] * c[0];
    const double dik = alpha * rikp / d[1] * c[1];
    for (int i = 0; i < size; ++i) {
      double fr = 0, dj = 0, dk = 0;  // radial factor and its derivative multipliers
      switch (phi) {
        case PA_GAUSS: fr = std::exp(-ietap[i] * (rijp + rikp)); dj = ietap[i]; dk = ietap[i]; break;
        case PA_IPOWP: {
          const double denij = 1.0 / (1.0 + ietap[i] * rijp), denik = 1.0 / (1.0 + ietap[i] * rikp);
          fr = denij * denik; dj = ietap[i] * denij; dk = ietap[i] * denik;
        } break;
        case PA_IPOWS: { const double den = 1.0 / (1.0 + ietap[i] * (rijp + rikp)); fr = den; dj = ietap[i] * den; dk = dj; } break;
        case PA_SECHP: {
          const double sij = sech(ietap[i] * rijp), sik = sech(ietap[i] * rikp);
          fr = sij * sik; dj = ietap[i] * std::sqrt(1.0 - sij * sij); dk = ietap[i] * std::sqrt(1.0 - sik * sik);
        } break;
        case PA_SECHS: {
          const double s = sech(ietap[i] * (rijp + rikp));
          fr = s; dj = ietap[i] * std::sqrt(1.0 - s * s); dk = dj;
        } break;
        default: throw std::invalid_argument("BasisA::force: invalid symmetry function");
      }
      const double cw = std::fabs(0.5 * (1.0 + lambda[i] * cs));
      const double gangle = std::pow(cw, zeta[i] - 1.0) * dEdG[i] * fr;
      const double fangle = cw * gangle;
      phi_o -= 0.5 * zeta[i] * lambda[i] * cprod * gangle;
      eta_o[0] -= fangle * (-dij * dj + g[0]) * c[1];
      eta_o[1] -= fangle * (-dik * dk + g[1]) * c[0];
    }
    phi_o *= norm; eta_o[0] *= norm; eta_o[1] *= norm; eta_o[2] *= norm;
  }
  // Per function m the three values BasisA::force sums over functions, for a unit dE/dG_m:
  // phif[m] = -dG_m/dcos, e0[m] = -dG_m/dr_ij, e1[m] = -dG_m/dr_ik (the expressions of force,
  // basis_angular.cpp:456-640, and of BasisA::forcep, basis_angular.cpp:642-761, with the sign of force).
  void dfunc(double cs, const double d[3], double* phif, double* e0, double* e1) const {
    const double c[2] = {cut_func(d[0]), cut_func(d[1])};
    const double g[2] = {cut_grad(d[0]), cut_grad(d[1])};
    const double cprod = c[0] * c[1];
    const double rijp = powint(d[0], alpha), rikp = powint(d[1], alpha);
    const double dij = alpha * rijp / d[0] * c[0];
    const double dik = alpha * rikp / d[1] * c[1];
    for (int i = 0; i < size; ++i) {
      double fr = 0, dj = 0, dk = 0;
      switch (phi) {
        case PA_GAUSS: fr = std::exp(-ietap[i] * (rijp + rikp)); dj = ietap[i]; dk = ietap[i]; break;
        case PA_IPOWP: {
          const double denij = 1.0 / (1.0 + ietap[i] * rijp), denik = 1.0 / (1.0 + ietap[i] * rikp);
          fr = denij * denik; dj = ietap[i] * denij; dk = ietap[i] * denik;
        } break;
        case PA_IPOWS: { const double den = 1.0 / (1.0 + ietap[i] * (rijp + rikp)); fr = den; dj = ietap[i] * den; dk = dj; } break;
        case PA_SECHP: {
          const double sij = sech(ietap[i] * rijp), sik = sech(ietap[i] * rikp);
          fr = sij * sik; dj = ietap[i] * std::sqrt(1.0 - sij * sij); dk = ietap[i] * std::sqrt(1.0 - sik * sik);
        } break;
        case PA_SECHS: {
          const double sv = sech(ietap[i] * (rijp + rikp));
          fr = sv; dj = ietap[i] * std::sqrt(1.0 - sv * sv); dk = dj;
        } break;
        default: throw std::invalid_argument("BasisA::force: invalid symmetry function");
      }
      const double cw = std::fabs(0.5 * (1.0 + lambda[i] * cs));
      const double gangle = std::pow(cw, zeta[i] - 1.0) * fr;
      const double fangle = cw * gangle;
      phif[i] = -0.5 * zeta[i] * lambda[i] * cprod * gangle * norm;
      e0[i] = -fangle * (-dij * dj + g[0]) * c[1] * norm;
      e1[i] = -fangle * (-dik * dk + g[1]) * c[0] * norm;
    }
  }
};

// ---------------------------------------------------------------- network
enum Neuron { N_UNKNOWN = 0, N_LINEAR = 1, N_SIGMOID = 2, N_TANH = 3 };  // src/ml/nn.hpp:84-103 (subset)

struct ANN {
  int nin = 0, neuron = N_UNKNOWN;
  std::vector<int> nodes;                    // nodes per layer (hidden..., output)
  std::vector<double> inpw, inpb, outw, outb;
  std::vector<std::vector<double>> b;        // b[l][n]
  std::vector<std::vector<double>> w;        // w[l][row*cols+col], rows = nodes[l]
  int nlayer() const { return (int)nodes.size(); }
  int cols(int l) const { return l == 0 ? nin : nodes[l - 1]; }
  // activation: hidden layers use the neuron, the last layer is linear (src/ml/nn.cpp:1134-1137)
  static void act(int neuron, double z, double& a, double& d) {
    switch (neuron) {
      case N_LINEAR: a = z; d = 1.0; break;                               // AFFPBP::af_lin, nn.cpp:144-148
      case N_TANH: { const double t = std::tanh(z); a = t; d = 1.0 - t * t; } break;  // AFFPBP::af_tanh, nn.cpp:209-216
      case N_SIGMOID:                                                     // AFFPBP::af_sigmoid, nn.cpp:165-181
        if (z >= 0) { const double e = std::exp(-z), f = 1.0 / (1.0 + e); a = f; d = e * f * f; }
        else { const double e = std::exp(z), f = 1.0 / (1.0 + e); a = e * f; d = e * f * f; }
        break;
      default: throw std::invalid_argument("ANN: unsupported neuron");
    }
  }
  // ANN::fpbp (src/ml/nn.cpp:1215-1233) followed by DODZ::grad (src/ml/nn.cpp:1620-1628);
  // returns out[0], writes dodi row 0 into dedg (if not null).
  double fpbp(const double* inp, double* dedg) const {
    const int L = nlayer();
    std::vector<double> ins(nin);
    for (int k = 0; k < nin; ++k) ins[k] = inpw[k] * (inp[k] + inpb[k]);
    std::vector<std::vector<double>> a(L), dadz(L);
    for (int l = 0; l < L; ++l) {
      const int R = nodes[l], C = cols(l);
      const std::vector<double>& x = (l == 0) ? ins : a[l - 1];
      a[l].resize(R); dadz[l].resize(R);
      const int nl = (l == L - 1) ? N_LINEAR : neuron;
      for (int r = 0; r < R; ++r) {
        double z = b[l][r];
        for (int c = 0; c < C; ++c) z += w[l][(size_t)r * C + c] * x[c];
        act(nl, z, a[l][r], dadz[l][r]);
      }
    }
    const double out = outb[0] + a[L - 1][0] * outw[0];
    if (dedg) {
      // dodz_L = outw * dadz_L ; dodz_{l-1} = (dodz_l W_l) .* dadz_{l-1} ; dodi = (dodz_0 W_0) .* inpw
      std::vector<double> g(nodes[L - 1]);
      for (int r = 0; r < nodes[L - 1]; ++r) g[r] = (r == 0 ? outw[0] : 0.0) * dadz[L - 1][r];
      for (int l = L - 1; l >= 0; --l) {
        const int R = nodes[l], C = cols(l);
        std::vector<double> h(C, 0.0);
        for (int c = 0; c < C; ++c) {
          double s = 0;
          for (int r = 0; r < R; ++r) s += g[r] * w[l][(size_t)r * C + c];
          h[c] = s;
        }
        if (l > 0) { for (int c = 0; c < C; ++c) h[c] *= dadz[l - 1][c]; g.swap(h); }
        else { for (int c = 0; c < C; ++c) dedg[c] = h[c] * inpw[c]; }
      }
    }
    return out;
  }
  // second derivative of the activation from its value a (AFFPBP's d2adz2 for tanh, sigmoid, linear)
  static double act2(int neuron, double a) {
    switch (neuron) {
      case N_TANH: return -2.0 * a * (1.0 - a * a);
      case N_SIGMOID: return a * (1.0 - a) * (1.0 - 2.0 * a);
      default: return 0.0;
    }
  }
  // grad += d/d parameter of (u . d out / d inp) at inp: the parameter gradient of the force term
  // of the loss (the mixed second derivative D2ODZDI of src/ml/nn.cpp:1789-1890, contracted with
  // u).  Forward-mode tangent inpw .* u through the layers, then reverse mode over both the
  // primal and the tangent chain.  Exact: the inpw factor of the first-layer weight term is kept
  // (D2ODZDI::grad, nn.cpp:1854-1862, leaves it out).
  void force_param_grad(const double* inp, const double* u, double* grad) const {
    const int L = nlayer();
    std::vector<double> ins(nin), tin(nin);
    for (int k = 0; k < nin; ++k) { ins[k] = inpw[k] * (inp[k] + inpb[k]); tin[k] = inpw[k] * u[k]; }
    std::vector<std::vector<double>> a(L), ta(L), tz(L), d1(L);
    for (int l = 0; l < L; ++l) {
      const int R = nodes[l], C = cols(l);
      const std::vector<double>& x = (l == 0) ? ins : a[l - 1];
      const std::vector<double>& tx = (l == 0) ? tin : ta[l - 1];
      a[l].resize(R); ta[l].resize(R); tz[l].resize(R); d1[l].resize(R);
      const int nl = (l == L - 1) ? N_LINEAR : neuron;
      for (int r = 0; r < R; ++r) {
        double z = b[l][r], t = 0;
        for (int c = 0; c < C; ++c) { z += w[l][(size_t)r * C + c] * x[c]; t += w[l][(size_t)r * C + c] * tx[c]; }
        act(nl, z, a[l][r], d1[l][r]);
        tz[l][r] = t;
        ta[l][r] = d1[l][r] * t;
      }
    }
    // h = outw . tangent of the last layer; adjoints dt (of the tangent pre-activations) and dp
    // (of the primal pre-activations)
    std::vector<std::vector<double>> dt(L), dp(L);
    dt[L - 1].assign(nodes[L - 1], 0.0);
    dp[L - 1].assign(nodes[L - 1], 0.0);
    for (int r = 0; r < nodes[L - 1]; ++r) dt[L - 1][r] = outw[r] * d1[L - 1][r];  // linear: d1 = 1, act2 = 0
    for (int l = L - 1; l > 0; --l) {
      const int R = nodes[l], C = cols(l);
      dt[l - 1].assign(C, 0.0);
      dp[l - 1].assign(C, 0.0);
      for (int c = 0; c < C; ++c) {
        double st = 0, sp = 0;
        for (int r = 0; r < R; ++r) { st += w[l][(size_t)r * C + c] * dt[l][r]; sp += w[l][(size_t)r * C + c] * dp[l][r]; }
        dt[l - 1][c] = d1[l - 1][c] * st;
        dp[l - 1][c] = d1[l - 1][c] * sp + act2(neuron, a[l - 1][c]) * tz[l - 1][c] * st;
      }
    }
    int count = 0;
    for (int l = 0; l < L; ++l)
      for (int n = 0; n < nodes[l]; ++n) grad[count++] += dp[l][n];
    for (int l = 0; l < L; ++l) {
      const int R = nodes[l], C = cols(l);
      for (int m = 0; m < C; ++m) {
        const double x = (l > 0) ? a[l - 1][m] : ins[m];
        const double tx = (l > 0) ? ta[l - 1][m] : tin[m];
        for (int n = 0; n < R; ++n) grad[count++] += dp[l][n] * x + dt[l][n] * tx;
      }
    }
  }
  // parameters in the reference's order (ANN::size, Cost::grad)
  void get_params(double* p) const {
    int count = 0;
    for (int l = 0; l < nlayer(); ++l) for (int n = 0; n < nodes[l]; ++n) p[count++] = b[l][n];
    for (int l = 0; l < nlayer(); ++l)
      for (int m = 0; m < cols(l); ++m) for (int n = 0; n < nodes[l]; ++n) p[count++] = w[l][(size_t)n * cols(l) + m];
  }
  void set_params(const double* p) {
    int count = 0;
    for (int l = 0; l < nlayer(); ++l) for (int n = 0; n < nodes[l]; ++n) b[l][n] = p[count++];
    for (int l = 0; l < nlayer(); ++l)
      for (int m = 0; m < cols(l); ++m) for (int n = 0; n < nodes[l]; ++n) w[l][(size_t)n * cols(l) + m] = p[count++];
  }
  // ANN::size (src/ml/nn.cpp:899-905): biases of every layer, then weights
  int size() const {
    int s = 0;
    for (int l = 0; l < nlayer(); ++l) s += nodes[l] * (1 + cols(l));
    return s;
  }
  // Cost::grad (src/ml/nn.cpp:1554-1589) after ANN::fpbp: adds dcdo * d out / d parameter into
  // grad, parameters ordered as the reference stores them: bias(l, n) for every layer, then
  // weight(l, n, m) with m (the input) outer and n (the node) inner.
  void param_grad(const double* inp, double dcdo, double* grad) const {
    const int L = nlayer();
    std::vector<double> ins(nin);
    for (int k = 0; k < nin; ++k) ins[k] = inpw[k] * (inp[k] + inpb[k]);
    std::vector<std::vector<double>> a(L), dadz(L), dcdz(L);
    for (int l = 0; l < L; ++l) {
      const int R = nodes[l], C = cols(l);
      const std::vector<double>& x = (l == 0) ? ins : a[l - 1];
      a[l].resize(R); dadz[l].resize(R);
      const int nl = (l == L - 1) ? N_LINEAR : neuron;
      for (int r = 0; r < R; ++r) {
        double z = b[l][r];
        for (int c = 0; c < C; ++c) z += w[l][(size_t)r * C + c] * x[c];
        act(nl, z, a[l][r], dadz[l][r]);
      }
    }
    dcdz[L - 1].assign(nodes[L - 1], 0.0);
    for (int r = 0; r < nodes[L - 1]; ++r) dcdz[L - 1][r] = dcdo * outw[r] * dadz[L - 1][r];
    for (int l = L - 1; l > 0; --l) {
      const int R = nodes[l], C = cols(l);
      dcdz[l - 1].assign(C, 0.0);
      for (int c = 0; c < C; ++c) {
        double s = 0;
        for (int r = 0; r < R; ++r) s += w[l][(size_t)r * C + c] * dcdz[l][r];
        dcdz[l - 1][c] = s * dadz[l - 1][c];
      }
    }
    int count = 0;
    for (int l = 0; l < L; ++l)
      for (int n = 0; n < nodes[l]; ++n) grad[count++] += dcdz[l][n];
    for (int l = 0; l < L; ++l) {
      const int R = nodes[l], C = cols(l);
      for (int m = 0; m < C; ++m) {
        const double x = (l > 0) ? a[l - 1][m] : ins[m];
        for (int n = 0; n < R; ++n) grad[count++] += dcdz[l][n] * x;
      }
    }
  }
};

struct NNH {
  std::string name;
  double mass = 0, energy = 0;  // Type: energy() is the vacuum energy (0 when absent)
  bool has_mass = false, has_energy = false;
  int ntypes = 0, nInput = 0, nInputR = 0, nInputA = 0;
  std::vector<BasisR> basisR;   // per neighbour type
  std::vector<BasisA> basisA;   // LMat linear order
  std::vector<int> offsetR, offsetA;
  ANN nn;
  static int lidx(int i, int j) { return (i >= j) ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }  // LMat, src/math/lmat.hpp:43-67
  // NNH::init_input, src/nnp/nnh.cpp:95-121
  void init_input() {
    nInputR = 0;
    for (int i = 0; i < ntypes; ++i) nInputR += basisR[i].size;
    offsetR.assign(ntypes, 0);
    for (int i = 1; i < ntypes; ++i) offsetR[i] = offsetR[i - 1] + basisR[i - 1].size;
    nInputA = 0;
    for (int i = 0; i < ntypes; ++i) for (int j = i; j < ntypes; ++j) nInputA += basisA[lidx(j, i)].size;
    offsetA.assign(basisA.size(), 0);
    for (size_t i = 1; i < basisA.size(); ++i) offsetA[i] = offsetA[i - 1] + basisA[i - 1].size;
    nInput = nInputR + nInputA;
  }
};

struct NNP {
  double rc = 0;
  int ntypes = 0;
  std::vector<NNH> nnh;
  std::map<std::string, int> index;
};

// ---------------------------------------------------------------- text IO
// Token splitting on string::WS = " \r\t\n" (src/str/string.hpp:16)
static std::vector<std::string> toks(const std::string& line) {
  std::vector<std::string> t;
  std::string cur;
  for (char ch : line) {
    if (ch == ' ' || ch == '\r' || ch == '\t' || ch == '\n') { if (!cur.empty()) { t.push_back(cur); cur.clear(); } }
    else cur.push_back(ch);
  }
  if (!cur.empty()) t.push_back(cur);
  return t;
}
struct LineReader {
  FILE* f;
  std::string line;
  std::vector<std::string> next() {
    line.clear();
    int ch;
    while ((ch = std::fgetc(f)) != EOF) { if (ch == '\n') break; line.push_back((char)ch); }
    if (ch == EOF && line.empty()) throw std::runtime_error("NNP::read: unexpected end of file");
    return toks(line);
  }
};
static const std::string& at(const std::vector<std::string>& t, size_t i) {
  if (i >= t.size()) throw std::runtime_error("NNP::read: missing token");
  return t[i];
}
static int read_cutname(const std::string& s) {  // cutoff::Name::read, src/nnp/cutoff.cpp:42-47
  return s == "STEP" ? CUT_STEP : s == "COS" ? CUT_COS : s == "TANH" ? CUT_TANH : CUT_UNKNOWN;
}
static int read_cutnorm(const std::string& s) {  // cutoff::Norm::read, src/nnp/cutoff.cpp:15-19
  return s == "UNIT" ? NORM_UNIT : s == "VOL" ? NORM_VOL : NORM_UNKNOWN;
}
static const char* cutname_str(int c) { return c == CUT_STEP ? "STEP" : c == CUT_COS ? "COS" : c == CUT_TANH ? "TANH" : "UNKNOWN"; }
static const char* cutnorm_str(int c) { return c == NORM_UNIT ? "UNIT" : c == NORM_VOL ? "VOL" : "UNKNOWN"; }
static const char* phir_names[] = {"UNKNOWN", "GAUSSIAN", "TANH", "SOFTPLUS", "LOGCOSH", "SWISH", "MISH"};
static const char* phia_names[] = {"UNKNOWN", "GAUSS", "IPOWP", "IPOWS", "SECHP", "SECHS"};
static int read_phir(const std::string& s) { for (int i = 1; i < 7; ++i) if (s == phir_names[i]) return i; return PR_UNKNOWN; }
static int read_phia(const std::string& s) { for (int i = 1; i < 6; ++i) if (s == phia_names[i]) return i; return PA_UNKNOWN; }

// BasisR::read, src/nnp/basis_radial.cpp:123-144
static void read_basisR(LineReader& lr, BasisR& b) {
  auto t = lr.next();
  const int nrm = read_cutnorm(at(t, 1)), name = read_cutname(at(t, 2));
  const double rc = std::atof(at(t, 3).c_str());
  const int phi = read_phir(at(t, 4));
  const int size = std::atoi(at(t, 5).c_str());
  if (phi == PR_UNKNOWN) throw std::invalid_argument("BasisR: invalid radial function type");
  b = BasisR();
  b.init(rc, name, nrm);
  b.phi = phi; b.size = size; b.rs.resize(size); b.eta.resize(size);
  for (int i = 0; i < size; ++i) {
    auto p = lr.next();
    b.rs[i] = std::atof(at(p, 0).c_str());
    b.eta[i] = std::atof(at(p, 1).c_str());
  }
}
// BasisA::read, src/nnp/basis_angular.cpp:113-138
static void read_basisA(LineReader& lr, BasisA& b) {
  auto t = lr.next();
  const int nrm = read_cutnorm(at(t, 1)), name = read_cutname(at(t, 2));
  const double rc = std::atof(at(t, 3).c_str());
  const int phi = read_phia(at(t, 4));
  const int size = std::atoi(at(t, 5).c_str());
  const int alpha = std::atoi(at(t, 6).c_str());
  if (phi == PA_UNKNOWN) throw std::invalid_argument("BasisA: invalid angular function type");
  b = BasisA();
  b.init(rc, name, nrm);
  b.phi = phi; b.size = size; b.alpha = alpha;
  b.eta.resize(size); b.zeta.resize(size); b.lambda.resize(size);
  for (int i = 0; i < size; ++i) {
    auto p = lr.next();
    b.eta[i] = std::atof(at(p, 0).c_str());
    b.zeta[i] = std::atof(at(p, 1).c_str());
    b.lambda[i] = std::atoi(at(p, 2).c_str());
  }
  b.init_ietap();
}
static int read_neuron(const std::string& s) {  // Neuron::read, src/ml/nn.cpp:115-134 (subset)
  return s == "LINEAR" ? N_LINEAR : s == "TANH" ? N_TANH : s == "SIGMOID" ? N_SIGMOID : N_UNKNOWN;
}
// ANN::read, src/ml/nn.cpp:1349-1425
static void read_ann(LineReader& lr, ANN& nn) {
  auto t = lr.next();
  std::vector<int> nodes;
  for (size_t i = 1; i < t.size(); ++i) nodes.push_back(std::atoi(t[i].c_str()));
  if (nodes.size() < 2) throw std::invalid_argument("ANN::read: invalid configuration");
  auto tn = lr.next();
  nn = ANN();
  nn.neuron = read_neuron(at(tn, 1));
  if (nn.neuron == N_UNKNOWN) throw std::invalid_argument("ANN::read: unsupported or invalid neuron " + at(tn, 1));
  nn.nin = nodes[0];
  nn.nodes.assign(nodes.begin() + 1, nodes.end());
  const int nout = nn.nodes.back();
  auto rdvec = [&](std::vector<double>& v, int n) {
    auto p = lr.next();
    v.resize(n);
    for (int i = 0; i < n; ++i) v[i] = std::atof(at(p, i + 1).c_str());
  };
  rdvec(nn.inpw, nn.nin);
  rdvec(nn.outw, nout);
  rdvec(nn.inpb, nn.nin);
  rdvec(nn.outb, nout);
  const int L = nn.nlayer();
  nn.b.resize(L); nn.w.resize(L);
  for (int l = 0; l < L; ++l) rdvec(nn.b[l], nn.nodes[l]);
  for (int l = 0; l < L; ++l) rdvec(nn.w[l], nn.nodes[l] * nn.cols(l));
}
// Type::read, src/nnp/type.cpp:32-70 (tags NAME, MASS, ENERGY used on this path; others skipped)
static void read_type(const std::vector<std::string>& t, NNH& h) {
  for (size_t i = 0; i < t.size(); ++i) {
    std::string tag = t[i];
    if (tag.size() && tag[0] == '#') break;
    for (auto& ch : tag) ch = (char)std::toupper((unsigned char)ch);
    if (tag == "NAME" && i + 1 < t.size()) h.name = t[++i];
    else if (tag == "MASS" && i + 1 < t.size()) { h.has_mass = true; h.mass = std::atof(t[++i].c_str()); }
    else if (tag == "ENERGY" && i + 1 < t.size()) { h.has_energy = true; h.energy = std::atof(t[++i].c_str()); }
    else if ((tag == "CHARGE" || tag == "CHI" || tag == "ETA" || tag == "JS" || tag == "C6" || tag == "RVDW" ||
              tag == "RCOV") && i + 1 < t.size()) ++i;
  }
}
// NNP::read, src/nnp/nnp.cpp:244-308
static void read_nnp(const char* path, NNP& nnp) {
  FILE* f = std::fopen(path, "r");
  if (!f) throw std::runtime_error(std::string("NNP::read: could not open nnp file: \"") + path + "\"");
  LineReader lr{f, {}};
  try {
    lr.next();  // header
    auto t = lr.next();
    const int ntypes = std::atoi(at(t, 1).c_str());
    if (ntypes <= 0) throw std::invalid_argument("NNP::read: invalid number of types");
    nnp = NNP();
    nnp.ntypes = ntypes;
    nnp.nnh.resize(ntypes);
    for (int n = 0; n < ntypes; ++n) {
      read_type(lr.next(), nnp.nnh[n]);
      nnp.index[nnp.nnh[n].name] = n;
    }
    for (int n = 0; n < ntypes; ++n) {
      NNH& h = nnp.nnh[n];
      h.ntypes = ntypes;
      h.basisR.resize(ntypes);
      h.basisA.resize(ntypes * (ntypes + 1) / 2);
    }
    t = lr.next();
    const double rc = std::atof(at(t, 1).c_str());
    if (rc <= 0) throw std::invalid_argument("NNP::read: invalid cutoff");
    nnp.rc = rc;
    auto idx = [&](const std::string& s) {
      auto it = nnp.index.find(s);
      if (it == nnp.index.end()) throw std::invalid_argument("NNP::read: unknown type " + s);
      return it->second;
    };
    for (int i = 0; i < ntypes; ++i) {
      const int II = idx(at(lr.next(), 1));
      for (int j = 0; j < ntypes; ++j) {
        const int JJ = idx(at(lr.next(), 1));
        read_basisR(lr, nnp.nnh[II].basisR[JJ]);
      }
      for (int j = 0; j < ntypes; ++j)
        for (int k = j; k < ntypes; ++k) {
          auto tt = lr.next();
          const int JJ = idx(at(tt, 1)), KK = idx(at(tt, 2));
          read_basisA(lr, nnp.nnh[II].basisA[NNH::lidx(JJ, KK)]);
        }
    }
    for (int i = 0; i < ntypes; ++i) nnp.nnh[i].init_input();
    for (int n = 0; n < ntypes; ++n) {
      const int II = idx(at(lr.next(), 1));
      read_ann(lr, nnp.nnh[II].nn);
      if (nnp.nnh[II].nn.nin != nnp.nnh[II].nInput)
        throw std::invalid_argument("NNP::read: network input size does not match the basis");
    }
  } catch (...) {
    std::fclose(f);
    throw;
  }
  std::fclose(f);
}
// NNP::write, src/nnp/nnp.cpp:198-237 (with Type::write type.cpp:125-137, BasisR::write
// basis_radial.cpp:107-116, BasisA::write basis_angular.cpp:97-106, ANN::write nn.cpp:1284-1324)
static void write_nnp(const char* path, const NNP& nnp) {
  FILE* w = std::fopen(path, "w");
  if (!w) throw std::runtime_error("NNP::write: could not open file");
  static const char* neuron_names[] = {"UNKNOWN", "LINEAR", "SIGMOID", "TANH"};
  std::fprintf(w, "ann\n");
  std::fprintf(w, "ntypes %i\n", nnp.ntypes);
  for (const NNH& h : nnp.nnh) {
    std::fprintf(w, "name %s ", h.name.c_str());
    if (h.has_mass) std::fprintf(w, "mass %f ", h.mass);
    if (h.has_energy) std::fprintf(w, "energy %f ", h.energy);
    std::fprintf(w, "\n");
  }
  std::fprintf(w, "rc %f\n", nnp.rc);
  for (int i = 0; i < nnp.ntypes; ++i) {
    const NNH& h = nnp.nnh[i];
    std::fprintf(w, "basis %s\n", h.name.c_str());
    for (int j = 0; j < nnp.ntypes; ++j) {
      const BasisR& b = h.basisR[j];
      std::fprintf(w, "basis_radial %s\n", nnp.nnh[j].name.c_str());
      std::fprintf(w, "BasisR %s %s %f %s %i\n", cutnorm_str(b.cutnorm), cutname_str(b.cutname), b.rc, phir_names[b.phi], b.size);
      for (int n = 0; n < b.size; ++n) std::fprintf(w, "\t%f %f\n", b.rs[n], b.eta[n]);
    }
    for (int j = 0; j < nnp.ntypes; ++j)
      for (int k = j; k < nnp.ntypes; ++k) {
        const BasisA& b = h.basisA[NNH::lidx(j, k)];
        std::fprintf(w, "basis_angular %s %s\n", nnp.nnh[j].name.c_str(), nnp.nnh[k].name.c_str());
        std::fprintf(w, "BasisA %s %s %f %s %i %i\n", cutnorm_str(b.cutnorm), cutname_str(b.cutname), b.rc, phia_names[b.phi], b.size, b.alpha);
        for (int n = 0; n < b.size; ++n) std::fprintf(w, "\t%f %f %i\n", b.eta[n], b.zeta[n], b.lambda[n]);
      }
  }
  for (int n = 0; n < nnp.ntypes; ++n) {
    const ANN& nn = nnp.nnh[n].nn;
    std::fprintf(w, "nn %s\n", nnp.nnh[n].name.c_str());
    std::fprintf(w, "nn %i ", nn.nin);
    for (int x : nn.nodes) std::fprintf(w, "%i ", x);
    std::fprintf(w, "\nneuron %s\n", neuron_names[nn.neuron]);
    std::fprintf(w, "inpw "); for (double x : nn.inpw) std::fprintf(w, "%.15f ", x);
    std::fprintf(w, "\noutw "); for (double x : nn.outw) std::fprintf(w, "%.15f ", x);
    std::fprintf(w, "\ninpb "); for (double x : nn.inpb) std::fprintf(w, "%.15f ", x);
    std::fprintf(w, "\noutb "); for (double x : nn.outb) std::fprintf(w, "%.15f ", x);
    std::fprintf(w, "\n");
    for (int l = 0; l < nn.nlayer(); ++l) {
      std::fprintf(w, "bias[%i] ", l + 1);
      for (double x : nn.b[l]) std::fprintf(w, "%.15f ", x);
      std::fprintf(w, "\n");
    }
    for (int l = 0; l < nn.nlayer(); ++l) {
      std::fprintf(w, "weight[%i,%i] ", l, l + 1);
      for (double x : nn.w[l]) std::fprintf(w, "%.15f ", x);
      std::fprintf(w, "\n");
    }
  }
  std::fclose(w);
}

// ---------------------------------------------------------------- structure / cell / neighbours
struct Cell {
  double R[9];     // column-major: R[3*c+r]
  double RInv[9];
  double dMax2 = 0;
  V3 shifts[6];
  bool periodic = false;
  V3 col(int c) const { return V3{R[3 * c], R[3 * c + 1], R[3 * c + 2]}; }
  // Cell::init, src/struc/cell.cpp:45-70 (3x3 inverse by cofactors)
  void init(const double* cell) {
    double fro = 0;
    for (int i = 0; i < 9; ++i) { R[i] = cell ? cell[i] : 0.0; fro += R[i] * R[i]; }
    periodic = std::sqrt(fro) > 0;
    if (!periodic) return;
    auto m = [&](int r, int c) { return R[3 * c + r]; };
    const double c00 = m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1);
    const double c01 = m(1, 2) * m(2, 0) - m(1, 0) * m(2, 2);
    const double c02 = m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0);
    const double det = m(0, 0) * c00 + m(0, 1) * c01 + m(0, 2) * c02;
    if (det == 0) throw std::invalid_argument("Cell::init: singular lattice");
    const double id = 1.0 / det;
    double inv[3][3];
    inv[0][0] = c00 * id;
    inv[1][0] = c01 * id;
    inv[2][0] = c02 * id;
    inv[0][1] = (m(0, 2) * m(2, 1) - m(0, 1) * m(2, 2)) * id;
    inv[1][1] = (m(0, 0) * m(2, 2) - m(0, 2) * m(2, 0)) * id;
    inv[2][1] = (m(0, 1) * m(2, 0) - m(0, 0) * m(2, 1)) * id;
    inv[0][2] = (m(0, 1) * m(1, 2) - m(0, 2) * m(1, 1)) * id;
    inv[1][2] = (m(0, 2) * m(1, 0) - m(0, 0) * m(1, 2)) * id;
    inv[2][2] = (m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0)) * id;
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) RInv[3 * c + r] = inv[r][c];
    double dmax = nrm(col(0));
    for (int i = 1; i < 3; ++i) { const double n = nrm(col(i)); if (n < dmax) dmax = n; }
    dmax *= 0.5;
    dMax2 = dmax * dmax;
    for (int c = 0; c < 3; ++c) {
      shifts[2 * c] = col(c);
      shifts[2 * c + 1] = V3{-R[3 * c], -R[3 * c + 1], -R[3 * c + 2]};
    }
  }
  static V3 mul(const double* M, const V3& v) {
    V3 o;
    for (int r = 0; r < 3; ++r) o[r] = M[r] * v[0] + M[3 + r] * v[1] + M[6 + r] * v[2];
    return o;
  }
  // Cell::diff, src/struc/cell.cpp:103-128.  Also returns the integer translation D with
  // diff = (v1 - v2) - R*D.
  V3 diff(const V3& v1, const V3& v2, int D[3]) const {
    const V3 d{v1[0] - v2[0], v1[1] - v2[1], v1[2] - v2[2]};
    V3 f = mul(RInv, d);
    for (int k = 0; k < 3; ++k) {
      const double fm = modlim(f[k], -0.5, 0.5);
      D[k] = (int)std::llround(f[k] - fm);
      f[k] = fm;
    }
    V3 out = mul(R, f);
    if (sqn(out) > dMax2) {
      V3 rmin = out;
      double dmin2 = sqn(rmin);
      int best = -1;
      for (int i = 0; i < 6; ++i) {
        const V3 t{out[0] + shifts[i][0], out[1] + shifts[i][1], out[2] + shifts[i][2]};
        const double d2 = sqn(t);
        if (d2 < dmin2) { dmin2 = d2; rmin = t; best = i; }
      }
      if (best >= 0) D[best / 2] += (best % 2 == 0) ? -1 : 1;
      out = rmin;
    }
    return out;
  }
};

struct Nb {
  V3 r;
  double dr;
  int index;
  bool min;
  int T[3];
};

// NeighborList::build(const Structure&, double rc), src/struc/neighbor.cpp:59-171; with centres,
// NeighborList::build(const Structure&, double rc, const std::vector<int>& subset)
// (src/struc/neighbor.cpp:283-394): only the listed atoms' lists, each scanning every atom.
static void build_neighbors(const Cell& cell, int natoms, const V3* posn, double rc, std::vector<std::vector<Nb>>& out,
                            const std::vector<int>* centres = nullptr) {
  out.assign(natoms, {});
  const int ncentre = centres ? (int)centres->size() : natoms;
  const double rc2 = rc * rc;
  if (cell.periodic) {
    // lattice vectors sorted from largest to smallest norm (std::sort on 3 elements is an
    // insertion sort in libstdc++, i.e. stable for equal norms)
    int perm[3] = {0, 1, 2};
    std::stable_sort(perm, perm + 3, [&](int a, int b) { return nrm(cell.col(a)) > nrm(cell.col(b)); });
    V3 Rv[3] = {cell.col(perm[0]), cell.col(perm[1]), cell.col(perm[2])};
    int shell[3];
    const V3 c01 = cross(Rv[0], Rv[1]);
    shell[0] = (int)std::floor(2.0 * rc / nrm(Rv[0]));
    shell[1] = (int)std::floor(2.0 * rc / (nrm(c01) / nrm(Rv[0])));
    shell[2] = (int)std::floor(2.0 * rc / std::fabs(dot(Rv[2], c01) / (nrm(Rv[0]) * nrm(Rv[1]))));
    struct Img { V3 v; int n[3]; };
    std::vector<Img> R_;
    for (int i = -shell[0]; i <= shell[0]; ++i)
      for (int j = -shell[1]; j <= shell[1]; ++j)
        for (int k = -shell[2]; k <= shell[2]; ++k) {
          Img im;
          for (int x = 0; x < 3; ++x) im.v[x] = i * Rv[0][x] + j * Rv[1][x] + k * Rv[2][x];
          im.n[perm[0]] = i; im.n[perm[1]] = j; im.n[perm[2]] = k;
          R_.push_back(im);
        }
    double fro = 0;
    for (int i = 0; i < 9; ++i) fro += cell.R[i] * cell.R[i];
    fro = std::sqrt(fro);
    for (int ci = 0; ci < ncentre; ++ci) {
      const int i = centres ? (*centres)[ci] : ci;
      for (int j = 0; j < natoms; ++j) {
        std::vector<Nb> nj;
        int D[3];
        const V3 rIJ = cell.diff(posn[i], posn[j], D);
        for (const Img& im : R_) {
          const V3 t{rIJ[0] - im.v[0], rIJ[1] - im.v[1], rIJ[2] - im.v[2]};
          const double d2 = sqn(t);
          const bool keep = (j != i) ? (d2 <= rc2) : (ZERO < d2 && d2 <= rc2);
          if (keep) {
            Nb nb;
            nb.r = t; nb.dr = std::sqrt(d2); nb.index = j; nb.min = false;
            for (int x = 0; x < 3; ++x) nb.T[x] = D[x] + im.n[x];
            nj.push_back(nb);
          }
        }
        if (j != i && !nj.empty()) {
          double mn = fro;
          int loc = -1;
          for (size_t n = 0; n < nj.size(); ++n)
            if (nj[n].dr < mn) { mn = nj[n].dr; loc = (int)n; }
          if (loc >= 0) nj[loc].min = true;
        }
        for (auto& nb : nj) out[i].push_back(nb);
      }
    }
  } else {
    for (int ci = 0; ci < ncentre; ++ci) {
      const int i = centres ? (*centres)[ci] : ci;
      for (int j = 0; j < natoms; ++j) {
        const V3 t{posn[i][0] - posn[j][0], posn[i][1] - posn[j][1], posn[i][2] - posn[j][2]};
        const double d2 = sqn(t);
        if (ZERO < d2 && d2 <= rc2) {
          Nb nb;
          nb.r = t; nb.dr = std::sqrt(d2); nb.index = j; nb.min = false;  // Neighbor() default min=false
          nb.T[0] = nb.T[1] = nb.T[2] = 0;
          out[i].push_back(nb);
        }
      }
    }
  }
}

// NNP::symm, src/nnp/nnp.cpp:334-381 (with centres: those atoms only)
static void symm(NNP& nnp, int natoms, const int* type, const std::vector<std::vector<Nb>>& nl, std::vector<std::vector<double>>& G,
                 const std::vector<int>* centres = nullptr) {
  G.assign(natoms, {});
  const int ncentre = centres ? (int)centres->size() : natoms;
  for (int ci = 0; ci < ncentre; ++ci) {
    const int i = centres ? (*centres)[ci] : ci;
    const NNH& h = nnp.nnh[type[i]];
    G[i].assign(h.nInput, 0.0);
    const std::vector<Nb>& L = nl[i];
    for (size_t j = 0; j < L.size(); ++j) {
      const int JJ = type[L[j].index];
      const V3& rIJ = L[j].r;
      const double dIJ = L[j].dr;
      h.basisR[JJ].symm_add(dIJ, G[i].data() + h.offsetR[JJ]);
      for (size_t k = j + 1; k < L.size(); ++k) {
        const int KK = type[L[k].index];
        const V3& rIK = L[k].r;
        const double dIK = L[k].dr;
        const V3 djk{rIK[0] - rIJ[0], rIK[1] - rIJ[1], rIK[2] - rIJ[2]};
        const double dJK = nrm(djk);
        const double cosIJK = dot(rIJ, rIK) / (dIJ * dIK);
        const double d[3] = {dIJ, dIK, dJK};
        const int off = h.nInputR + h.offsetA[NNH::lidx(JJ, KK)];
        h.basisA[NNH::lidx(JJ, KK)].symm_add(cosIJK, d, G[i].data() + off);
      }
    }
  }
}

// NNP::force (src/nnp/nnp.cpp:416-482) and NNP::compute (src/nnp/nnp.cpp:496-566):
// both run one fpbp per atom then the same chain rule; compute also sums the network outputs.
static double force(NNP& nnp, int natoms, const int* type, const std::vector<std::vector<Nb>>& nl,
                    const std::vector<std::vector<double>>& G, std::vector<V3>& F, const std::vector<int>* centres = nullptr) {
  F.assign(natoms, V3{0, 0, 0});
  double energy = 0;
  const int ncentre = centres ? (int)centres->size() : natoms;
  for (int ci = 0; ci < ncentre; ++ci) {
    const int i = centres ? (*centres)[ci] : ci;
    const NNH& h = nnp.nnh[type[i]];
    std::vector<double> dEdG(h.nInput);
    energy += h.nn.fpbp(G[i].data(), dEdG.data());
    const std::vector<Nb>& L = nl[i];
    for (size_t j = 0; j < L.size(); ++j) {
      const int JJ = type[L[j].index];
      const int jj = L[j].index;
      const bool jmin = L[j].min;
      const V3& rIJ = L[j].r;
      const double dIJ = L[j].dr, dIJi = 1.0 / dIJ;
      {
        const double amp = h.basisR[JJ].force(dIJ, dEdG.data() + h.offsetR[JJ]) * dIJi;
        for (int x = 0; x < 3; ++x) F[i][x] += amp * rIJ[x];
        if (jmin) for (int x = 0; x < 3; ++x) F[jj][x] -= amp * rIJ[x];
      }
      for (size_t k = j + 1; k < L.size(); ++k) {
        const int KK = type[L[k].index];
        const int kk = L[k].index;
        const bool kmin = L[k].min;
        const V3& rIK = L[k].r;
        const double dIK = L[k].dr, dIKi = 1.0 / dIK;
        const V3 rJK{rIK[0] - rIJ[0], rIK[1] - rIJ[1], rIK[2] - rIJ[2]};
        const double dJK = nrm(rJK), dJKi = 1.0 / dJK;
        const int lk = NNH::lidx(JJ, KK);
        const int off = h.nInputR + h.offsetA[lk];
        double phi = 0, eta[3] = {0, 0, 0};
        const double cosIJK = dot(rIJ, rIK) * dIJi * dIKi;
        const double d[3] = {dIJ, dIK, dJK};
        h.basisA[lk].force(phi, eta, cosIJK, d, dEdG.data() + off);
        const double ai = (phi * (dIKi - cosIJK * dIJi) + eta[0]) * dIJi;
        const double bi = (phi * (dIJi - cosIJK * dIKi) + eta[1]) * dIKi;
        for (int x = 0; x < 3; ++x) F[i][x] += ai * rIJ[x];
        for (int x = 0; x < 3; ++x) F[i][x] += bi * rIK[x];
        if (jmin) {
          for (int x = 0; x < 3; ++x) F[jj][x] -= (-phi * cosIJK * dIJi + eta[0]) * rIJ[x] * dIJi + phi * dIJi * rIK[x] * dIKi;
          for (int x = 0; x < 3; ++x) F[jj][x] -= eta[2] * rJK[x] * dJKi;
        }
        if (kmin) {
          for (int x = 0; x < 3; ++x) F[kk][x] -= (-phi * cosIJK * dIKi + eta[1]) * rIK[x] * dIKi + phi * dIKi * rIJ[x] * dIJi;
          for (int x = 0; x < 3; ++x) F[kk][x] += eta[2] * rJK[x] * dJKi;
        }
      }
    }
  }
  return energy;
}

// u_i[f] = sum_k t_k . C_ifk, where C_ifk is the force on atom k per unit dE/dG_if in NNP::force
// (nnp.cpp:416-482, minimum-image rule included): the descriptor-space weights of the force
// term of the loss, t_k = dloss/dF_k.
static void force_tangent(NNP& nnp, int natoms, const int* type, const std::vector<std::vector<Nb>>& nl, const std::vector<V3>& t,
                          std::vector<std::vector<double>>& u) {
  u.assign(natoms, {});
  for (int i = 0; i < natoms; ++i) {
    const NNH& h = nnp.nnh[type[i]];
    u[i].assign(h.nInput, 0.0);
    const std::vector<Nb>& L = nl[i];
    std::vector<double> dv(64), pf(64), e0(64), e1(64);
    for (size_t j = 0; j < L.size(); ++j) {
      const int JJ = type[L[j].index];
      const int jj = L[j].index;
      const bool jmin = L[j].min;
      const V3& rIJ = L[j].r;
      const double dIJ = L[j].dr, dIJi = 1.0 / dIJ;
      {
        const BasisR& bR = h.basisR[JJ];
        dv.resize(std::max(bR.size, 1));
        bR.dval(dIJ, dv.data());
        // amp_m = -dG_m/dr / r: F_i += amp rIJ, F_j -= amp rIJ (minimum image only)
        const double proj = dot(t[i], rIJ) - (jmin ? dot(t[jj], rIJ) : 0.0);
        for (int m = 0; m < bR.size; ++m) u[i][h.offsetR[JJ] + m] += -dv[m] * dIJi * proj;
      }
      for (size_t k = j + 1; k < L.size(); ++k) {
        const int KK = type[L[k].index];
        const int kk = L[k].index;
        const bool kmin = L[k].min;
        const V3& rIK = L[k].r;
        const double dIK = L[k].dr, dIKi = 1.0 / dIK;
        const V3 rJK{rIK[0] - rIJ[0], rIK[1] - rIJ[1], rIK[2] - rIJ[2]};
        const double dJK = nrm(rJK);
        const int lk = NNH::lidx(JJ, KK);
        const BasisA& bA = h.basisA[lk];
        const int off = h.nInputR + h.offsetA[lk];
        const double cosIJK = dot(rIJ, rIK) * dIJi * dIKi;
        const double d[3] = {dIJ, dIK, dJK};
        const size_t n = std::max(bA.size, 1);
        pf.resize(n); e0.resize(n); e1.resize(n);
        bA.dfunc(cosIJK, d, pf.data(), e0.data(), e1.data());
        const double ti_j = dot(t[i], rIJ) * dIJi, ti_k = dot(t[i], rIK) * dIKi;
        const double tj_j = jmin ? dot(t[jj], rIJ) * dIJi : 0.0, tj_k = jmin ? dot(t[jj], rIK) * dIKi : 0.0;
        const double tk_j = kmin ? dot(t[kk], rIJ) * dIJi : 0.0, tk_k = kmin ? dot(t[kk], rIK) * dIKi : 0.0;
        for (int m = 0; m < bA.size; ++m) {
          const double phi = pf[m];
          // centre: (phi (1/dIK - cos/dIJ) + eta0) rIJ/dIJ + (phi (1/dIJ - cos/dIK) + eta1) rIK/dIK
          double v = (phi * (dIKi - cosIJK * dIJi) + e0[m]) * ti_j + (phi * (dIJi - cosIJK * dIKi) + e1[m]) * ti_k;
          // j: -[(-phi cos/dIJ + eta0) rIJ/dIJ + phi/dIJ rIK/dIK]; k likewise (eta2 = 0)
          v -= (-phi * cosIJK * dIJi + e0[m]) * tj_j + phi * dIJi * tj_k;
          v -= (-phi * cosIJK * dIKi + e1[m]) * tk_k + phi * dIKi * tk_j;
          u[i][off + m] += v;
        }
      }
    }
  }
}

}  // namespace orc

// ---------------------------------------------------------------- C interface
using namespace orc;

static void set_err(char* err, int errlen, const char* msg) {
  if (err && errlen > 0) { std::strncpy(err, msg, errlen - 1); err[errlen - 1] = 0; }
}

extern "C" void* oracle_nnp_read(const char* path, char* err, int errlen) {
  try {
    NNP* n = new NNP();
    try { read_nnp(path, *n); } catch (...) { delete n; throw; }
    return n;
  } catch (std::exception& e) {
    set_err(err, errlen, e.what());
    return nullptr;
  }
}
extern "C" void oracle_nnp_free(void* nnp) { delete (NNP*)nnp; }
extern "C" int oracle_nnp_ntypes(const void* nnp) { return ((const NNP*)nnp)->ntypes; }
extern "C" int oracle_nnp_ninput(const void* nnp, int type) { return ((const NNP*)nnp)->nnh[type].nInput; }
extern "C" double oracle_nnp_rc(const void* nnp) { return ((const NNP*)nnp)->rc; }
extern "C" int oracle_nnp_type_index(const void* nnp, const char* name) {
  const NNP* n = (const NNP*)nnp;
  auto it = n->index.find(name);
  return it == n->index.end() ? -1 : it->second;
}
extern "C" int oracle_nnp_write(const void* nnp, const char* path) {
  try { write_nnp(path, *(const NNP*)nnp); return 0; } catch (...) { return -1; }
}

extern "C" int oracle_neighbors(double rc, int natoms, const double* posn, const double* cellp, int cap,
                                int* count, int* index, double* r, double* dr, unsigned char* min, int* shift) {
  try {
    Cell cell;
    cell.init(cellp);
    std::vector<V3> p(natoms);
    for (int i = 0; i < natoms; ++i) p[i] = V3{posn[3 * i], posn[3 * i + 1], posn[3 * i + 2]};
    std::vector<std::vector<Nb>> nl;
    build_neighbors(cell, natoms, p.data(), rc, nl);
    int rc_ = 0;
    for (int i = 0; i < natoms; ++i) {
      count[i] = (int)nl[i].size();
      if (count[i] > cap) rc_ = -1;
      const int n = std::min(count[i], cap);
      for (int s = 0; s < n; ++s) {
        const size_t o = (size_t)i * cap + s;
        const Nb& nb = nl[i][s];
        if (index) index[o] = nb.index;
        if (r) for (int x = 0; x < 3; ++x) r[3 * o + x] = nb.r[x];
        if (dr) dr[o] = nb.dr;
        if (min) min[o] = nb.min ? 1 : 0;
        if (shift) for (int x = 0; x < 3; ++x) shift[3 * o + x] = nb.T[x];
      }
    }
    return rc_;
  } catch (...) {
    return -2;
  }
}

extern "C" int oracle_compute(void* nnpv, int natoms, const double* posn, const int* type, const double* cellp,
                              int flags, double* energy, double* force_out, double* symm_out, int symm_stride) {
  try {
    NNP& nnp = *(NNP*)nnpv;
    for (int i = 0; i < natoms; ++i)
      if (type[i] < 0 || type[i] >= nnp.ntypes) return -3;
    Cell cell;
    cell.init(cellp);
    std::vector<V3> p(natoms);
    for (int i = 0; i < natoms; ++i) p[i] = V3{posn[3 * i], posn[3 * i + 1], posn[3 * i + 2]};
    std::vector<std::vector<Nb>> nl;
    build_neighbors(cell, natoms, p.data(), nnp.rc, nl);
    std::vector<std::vector<double>> G;
    orc::symm(nnp, natoms, type, nl, G);
    if (symm_out)
      for (int i = 0; i < natoms; ++i)
        for (size_t k = 0; k < G[i].size(); ++k) symm_out[(size_t)i * symm_stride + k] = G[i][k];
    double e = 0;
    if (flags & ORACLE_ENERGY) {
      // NNP::energy: sum of network outputs plus the species vacuum energy (NNH::energy, nnh.cpp:127-130)
      for (int i = 0; i < natoms; ++i) {
        const NNH& h = nnp.nnh[type[i]];
        e += h.nn.fpbp(G[i].data(), nullptr) + h.energy;
      }
    }
    if (flags & (ORACLE_FORCE | ORACLE_COMPUTE)) {
      std::vector<V3> F;
      const double ec = orc::force(nnp, natoms, type, nl, G, F);
      if (flags & ORACLE_COMPUTE) e = ec;
      if (force_out)
        for (int i = 0; i < natoms; ++i) for (int x = 0; x < 3; ++x) force_out[3 * i + x] = F[i][x];
    }
    if (energy) *energy = e;
    return 0;
  } catch (...) {
    return -2;
  }
}

// The per-centre work of oracle_compute (E+F) for a subset of centre atoms: their neighbour
// lists (each scanning every atom, as NeighborList::build(struc, rc, subset) does), descriptors,
// network passes and chain rule.  Returns the centres' network outputs plus vacuum energies in
// *energy.  The cost per centre equals that of the full evaluation, so a sample of centres times
// the full structure's per-atom cost.
extern "C" int oracle_compute_centres(void* nnpv, int natoms, const double* posn, const int* type, const double* cellp, int ncentre,
                                      const int* centres, double* energy) {
  try {
    NNP& nnp = *(NNP*)nnpv;
    for (int i = 0; i < natoms; ++i)
      if (type[i] < 0 || type[i] >= nnp.ntypes) return -3;
    std::vector<int> sub(centres, centres + ncentre);
    for (int i : sub)
      if (i < 0 || i >= natoms) return -3;
    Cell cell;
    cell.init(cellp);
    std::vector<V3> p(natoms);
    for (int i = 0; i < natoms; ++i) p[i] = V3{posn[3 * i], posn[3 * i + 1], posn[3 * i + 2]};
    std::vector<std::vector<Nb>> nl;
    build_neighbors(cell, natoms, p.data(), nnp.rc, nl, &sub);
    std::vector<std::vector<double>> G;
    orc::symm(nnp, natoms, type, nl, G, &sub);
    std::vector<V3> F;
    double e = orc::force(nnp, natoms, type, nl, G, F, &sub);
    for (int i : sub) e += nnp.nnh[type[i]].energy;
    if (energy) *energy = e;
    return 0;
  } catch (...) {
    return -2;
  }
}

extern "C" double oracle_network(void* nnpv, int type, const double* symm, double* dedg) {
  NNP& nnp = *(NNP*)nnpv;
  return nnp.nnh[type].nn.fpbp(symm, dedg);
}

extern "C" int oracle_nnp_nparams(const void* nnp, int type) { return ((const NNP*)nnp)->nnh[type].nn.size(); }

// The per-batch error and gradient of the energy trainer (NNPTE::error, src/nnp/nnpte.cpp:870-921):
// per structure E = sum of atomic network outputs (no vacuum energies), dE = (E - E_ref)/N, the loss
// (0 MSE: dE^2/2, 1 MAE: |dE|, 2 HUBER: delta^2 (sqrt(1 + (dE/delta)^2) - 1), 3 ASINH:
// delta^2 (1 - sqrt(1 + x^2) + x asinh x) with x = dE/delta) and dc/dout = dloss/d(dE) / N;
// grad (concatenated per type, oracle_nnp_nparams each) += dc/dout * d out/d parameter summed over
// the structure's atoms (Cost::grad).  error[0] = sum of losses, error[1] = sum of dE^2.
// symm: the atoms' symmetry functions, one row of `stride` values per atom.
extern "C" int oracle_train_grad(void* nnpv, int nstruc, const int* natoms, const double* symm, int stride, const int* type,
                                 const double* eref, int loss, double delta, double* error, double* grad) {
  try {
    NNP& nnp = *(NNP*)nnpv;
    std::vector<size_t> goff(nnp.ntypes + 1, 0);
    for (int t = 0; t < nnp.ntypes; ++t) goff[t + 1] = goff[t] + nnp.nnh[t].nn.size();
    for (size_t k = 0; k < goff[nnp.ntypes]; ++k) grad[k] = 0.0;
    error[0] = error[1] = 0.0;
    size_t a0 = 0;
    for (int s = 0; s < nstruc; ++s) {
      double energy = 0;
      for (int n = 0; n < natoms[s]; ++n) {
        const size_t a = a0 + n;
        energy += nnp.nnh[type[a]].nn.fpbp(symm + a * stride, nullptr);
      }
      const double norm = 1.0 / natoms[s];
      const double dE = (energy - eref[s]) * norm;
      double dcdo = norm;
      switch (loss) {
        case 0: error[0] += 0.5 * dE * dE; dcdo *= dE; break;
        case 1: error[0] += std::fabs(dE); dcdo *= (dE > 0) ? 1.0 : ((dE < 0) ? -1.0 : 0.0); break;
        case 2: {
          const double arg = dE / delta, sq = std::sqrt(1.0 + arg * arg);
          error[0] += delta * delta * (sq - 1.0);
          dcdo *= dE / sq;
        } break;
        case 3: {
          const double arg = dE / delta, sq = std::sqrt(1.0 + arg * arg), lg = std::log(arg + sq);
          error[0] += delta * delta * (1.0 - sq + arg * lg);
          dcdo *= lg * delta;
        } break;
        default: return -1;
      }
      error[1] += dE * dE;
      for (int n = 0; n < natoms[s]; ++n) {
        const size_t a = a0 + n;
        nnp.nnh[type[a]].nn.param_grad(symm + a * stride, dcdo, grad + goff[type[a]]);
      }
      a0 += natoms[s];
    }
    return 0;
  } catch (...) {
    return -2;
  }
}

extern "C" void oracle_nnp_get_params(const void* nnpv, int type, double* p) { ((const NNP*)nnpv)->nnh[type].nn.get_params(p); }
extern "C" void oracle_nnp_set_params(void* nnpv, int type, const double* p) { ((NNP*)nnpv)->nnh[type].nn.set_params(p); }

// The force trainer's batch error and gradient: the loss of NNPTEF::error (src/nnp/nnptef.cpp:1043-1135)
//   sum_s loss(dE_s) + sum_atoms 0.5 beta |(F_nnp - F_ref) / N_s|^2,
// dE_s = (E_s - E_ref,s)/N_s with E_s the sum of network outputs (no vacuum energies) and F the
// forces of NNP::force (minimum-image rule), loss as in oracle_train_grad.  grad is the exact
// gradient of that loss: the energy term as in the energy trainer, the force term through
// u_i = sum_k t_k . dF_k/d(dE/dG_i) with t_k = beta (F_k - F_ref,k)/N_s^2 and the mixed second
// derivative of each atom's network (ANN::force_param_grad).  error[0] = the loss, error[1] =
// sum of dE^2, error[2] = sum over atoms of |(F_nnp - F_ref)/N_s|^2.
// posn/fref: concatenated N x 3; cells: nstruc x 9 column-major.
extern "C" int oracle_train_force_grad(void* nnpv, int nstruc, const int* natoms, const double* posn, const int* type, const double* cells,
                                       const double* eref, const double* fref, double beta, int loss, double delta, double* error,
                                       double* grad) {
  try {
    NNP& nnp = *(NNP*)nnpv;
    std::vector<size_t> goff(nnp.ntypes + 1, 0);
    for (int t = 0; t < nnp.ntypes; ++t) goff[t + 1] = goff[t] + nnp.nnh[t].nn.size();
    for (size_t k = 0; k < goff[nnp.ntypes]; ++k) grad[k] = 0.0;
    error[0] = error[1] = error[2] = 0.0;
    size_t a0 = 0;
    for (int s = 0; s < nstruc; ++s) {
      const int n = natoms[s];
      const int* ty = type + a0;
      for (int i = 0; i < n; ++i)
        if (ty[i] < 0 || ty[i] >= nnp.ntypes) return -3;
      Cell cell;
      cell.init(cells + 9 * (size_t)s);
      std::vector<V3> p(n);
      for (int i = 0; i < n; ++i) p[i] = V3{posn[3 * (a0 + i)], posn[3 * (a0 + i) + 1], posn[3 * (a0 + i) + 2]};
      std::vector<std::vector<Nb>> nl;
      build_neighbors(cell, n, p.data(), nnp.rc, nl);
      std::vector<std::vector<double>> G;
      orc::symm(nnp, n, ty, nl, G);
      std::vector<V3> F;
      const double energy = orc::force(nnp, n, ty, nl, G, F);
      const double norm = 1.0 / n;
      const double dE = (energy - eref[s]) * norm;
      double dcdo = norm;
      switch (loss) {
        case 0: error[0] += 0.5 * dE * dE; dcdo *= dE; break;
        case 1: error[0] += std::fabs(dE); dcdo *= (dE > 0) ? 1.0 : ((dE < 0) ? -1.0 : 0.0); break;
        case 2: {
          const double arg = dE / delta, sq = std::sqrt(1.0 + arg * arg);
          error[0] += delta * delta * (sq - 1.0);
          dcdo *= dE / sq;
        } break;
        case 3: {
          const double arg = dE / delta, sq = std::sqrt(1.0 + arg * arg), lg = std::log(arg + sq);
          error[0] += delta * delta * (1.0 - sq + arg * lg);
          dcdo *= lg * delta;
        } break;
        default: return -1;
      }
      error[1] += dE * dE;
      std::vector<V3> t(n);
      for (int i = 0; i < n; ++i) {
        double f2 = 0;
        for (int x = 0; x < 3; ++x) {
          const double fd = (F[i][x] - fref[3 * (a0 + i) + x]) * norm;
          f2 += fd * fd;
          t[i][x] = beta * fd * norm;
        }
        error[0] += 0.5 * beta * f2;
        error[2] += f2;
      }
      std::vector<std::vector<double>> u;
      force_tangent(nnp, n, ty, nl, t, u);
      for (int i = 0; i < n; ++i) {
        const ANN& nn = nnp.nnh[ty[i]].nn;
        nn.param_grad(G[i].data(), dcdo, grad + goff[ty[i]]);
        nn.force_param_grad(G[i].data(), u[i].data(), grad + goff[ty[i]]);
      }
      a0 += n;
    }
    return 0;
  } catch (...) {
    return -2;
  }
}
