// Oracle kit driver: runs the reference's unchanged generator, fitter and
// Minuit2 on seeded synthetic events and writes golden vectors as JSON.
//
// TEST INFRASTRUCTURE ONLY (built by oracle/Makefile into oracle/_ref/ from
// the reference sources where they lie; never shipped, never on the product
// path). Workloads:
//   mass  : fsig*Gauss(m; mb, sigma) + (1-fsig)*Exp(alpha*m) on m in
//           [5000,5600] (pdf.hh:139-194, :423-484, :486-651), 4 floating
//           parameters, fitter options of benchmarking/morefit_massfit.cc:77-99
//           but with analytic gradient and Hessian.
//   pwave : KstarmumuAngularPDF (physicspdfs.hh:28-214) on ctl, ctk in
//           [-1,1], phi in [-pi,pi], 8 floating parameters, fitter options of
//           benchmarking/morefit_kstarmumu.cc:74-92.
//   spwave: the P-wave density plus S-wave and S-P interference terms times
//           a Legendre acceptance (SPwaveAccPDF below), 14 floating parameters.
//   mass_w: the mass model with an event weight column (weighted fit with
//           the Fisher kernel and the covariance correction).
//   cbpoly: Crystal Ball + quadratic polynomial on x in [-1,1] (pdf.hh:199-419,
//           :717-892), 7 floating parameters.
// Events come from generator::generate on the accelerator path with one
// xoshiro128++ stream seeded by Xoshiro128pp::setSeed(229387429)
// (random.hh:355-362, generator.hh:102-113), as in the reference drivers.
//
// Usage:
//   refkit golden <workload> <nevents> <out.json> [events.bin]
//   refkit bench  <mass|pwave|spwave> <nevents> <nthreads> <nevals>
//   refkit toys   <pwave> <ntoys> <mean events> <jitter> <out.json> [seed]
//   refkit plot   <workload> <nevents> <variable> <nbins> <out.py> <out.json>
//   refkit fitfile <workload> <datasets.bin> <out.json>
#define MOREFIT_H 1  // keep graph.hh from pulling in the OpenCL/LLVM backends
#include <cassert>
#include <chrono>
#include <cmath>
#include <fstream>
#include <functional>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "graph.hh"
#include "eventvector.hh"
#include "parametervector.hh"
#include "pdf.hh"
#include "physicspdfs.hh"
#include "compute.hh"
#include "gcc_block.hh"
#include "fitter.hh"
#include "generator.hh"
#include "plotter.hh"
#include "random.hh"

using namespace morefit;
typedef double kT;
typedef double eT;
typedef LLVMBackend backendT;
typedef LLVMBlock<kT, eT> blockT;

// ---- capture hooks: every parameter vector and Kahan result, per kernel ----
struct Capture {
  std::map<std::string, std::vector<double>> params, sums, outputs;
};
static Capture* g_capture = nullptr;
static void install_capture() {
  block_observer() = [](const std::string& kernel, const char* what, const std::vector<double>& v) {
    if (!g_capture) return;
    const std::string w = what;
    if (w == "params")
      g_capture->params[kernel] = v;
    else if (w == "sums")
      g_capture->sums[kernel] = v;
    else
      g_capture->outputs[kernel] = v;
  };
}

static std::string jstr(const std::string& s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') {
      o += '\\';
      o += c;
    } else if (c == '\n') {
      o += "\\n";
    } else if (static_cast<unsigned char>(c) < 0x20) {
      char b[8];
      std::snprintf(b, sizeof b, "\\u%04x", unsigned(c));
      o += b;
    } else {
      o += c;
    }
  }
  return o + "\"";
}
static std::string jnum(double v) {
  if (std::isnan(v)) return "null";
  char b[64];
  std::snprintf(b, sizeof b, "%.17g", v);
  return b;
}
static std::string jvec(const std::vector<double>& v) {
  std::string o = "[";
  for (size_t i = 0; i < v.size(); i++) o += (i ? "," : "") + jnum(v[i]);
  return o + "]";
}
static std::string jsvec(const std::vector<std::string>& v) {
  std::string o = "[";
  for (size_t i = 0; i < v.size(); i++) o += (i ? "," : "") + jstr(v[i]);
  return o + "]";
}

static uint64_t fnv1a(const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  uint64_t h = 1469598103934665603ULL;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 1099511628211ULL;
  }
  return h;
}

// ---- S+P-wave K*mumu density with a Legendre angular acceptance ----------
// No counterpart in the reference: written here in the reference's own graph
// language (Constant / Variable / Sqrt / Cos / Sin nodes and the operators of
// graph.hh, as KstarmumuAngularPDF builds its density, physicspdfs.hh:39-77),
// so the reference's fitter hoists, differentiates and prints its kernels.
//   prob = sum_k c_k(theta) * (eps(Omega) f_k(Omega))
// with the 11 P-wave terms of KstarmumuAngularPDF scaled by (1 - FS), the
// S-wave term FS 3/(16 pi) sin^2(thl), and five S-P interference terms
//   AS  sin^2(thl) cos(thK),  AS4 sin(thK) sin(2thl) cos(phi),
//   AS5 sin(thK) sin(thl) cos(phi),  AS7 sin(thK) sin(thl) sin(phi),
//   AS8 sin(thK) sin(2thl) sin(phi)   (each times 9/(32 pi)),
// and eps = prod over x in {ctl, ctk, phi/pi} of (1 + sum_{l=1..4} a_{x,l} P_l(x)),
// a_{x,l} uniform in [-0.05, 0.05] from a fixed SplitMix64 stream.
// Every f_k and eps factor into functions of one angle, so
//   norm = sum_k c_k(theta) I_k,  I_k = prod over angles of 1D integrals,
// computed once with Gauss-Legendre quadrature (cos theta integrals in the
// angle, 256 nodes).
namespace spw {

struct Term {
  int g, h, u;   // one-angle factors: ctl, ctk, phi (indices below)
  double c;      // constant
  int coef;      // parameter-only coefficient (index below)
};
// ctl factors: 0 = 1, 1 = 2ctl^2-1, 2 = 1-ctl^2, 3 = 2 ctl sqrt(1-ctl^2), 4 = sqrt(1-ctl^2), 5 = ctl
// ctk factors: 0 = 1-ctk^2, 1 = ctk^2, 2 = 2 ctk sqrt(1-ctk^2), 3 = 1, 4 = ctk, 5 = sqrt(1-ctk^2)
// phi factors: 0 = 1, 1 = cos 2phi, 2 = cos phi, 3 = sin phi, 4 = sin 2phi
static double fl(int i, double x) {
  const double s = std::sqrt(std::max(0.0, 1.0 - x * x));
  switch (i) { case 0: return 1.0; case 1: return 2 * x * x - 1; case 2: return 1 - x * x; case 3: return 2 * x * s; case 4: return s; default: return x; }
}
static double fk(int i, double x) {
  const double s = std::sqrt(std::max(0.0, 1.0 - x * x));
  switch (i) { case 0: return 1 - x * x; case 1: return x * x; case 2: return 2 * x * s; case 3: return 1.0; case 4: return x; default: return s; }
}
static double fp(int i, double x) {
  switch (i) { case 0: return 1.0; case 1: return std::cos(2 * x); case 2: return std::cos(x); case 3: return std::sin(x); default: return std::sin(2 * x); }
}
static const double C9 = 9.0 / 32.0 / M_PI;
// coefficient index: 0 (1-FS)3/4(1-Fl), 1 (1-FS)Fl, 2 (1-FS)1/4(1-Fl), 3 (1-FS)(-Fl), 4..10 (1-FS)*{S3,S4,S5,4/3 Afb,S7,S8,S9},
// 11 FS, 12 AS, 13 AS4, 14 AS5, 15 AS7, 16 AS8
static const Term TERMS[17] = {
    {0, 0, 0, C9, 0},      {0, 1, 0, C9, 1},  {1, 0, 0, C9, 2},  {1, 1, 0, C9, 3},  {2, 0, 1, C9, 4},
    {3, 2, 2, C9, 5},      {4, 2, 2, C9, 6},  {5, 0, 0, C9, 7},  {4, 2, 3, C9, 8},  {3, 2, 3, C9, 9},
    {2, 0, 4, C9, 10},     {2, 3, 0, 3.0 / 16.0 / M_PI, 11},   {2, 4, 0, C9, 12}, {3, 5, 2, C9, 13},
    {4, 5, 2, C9, 14},     {4, 5, 3, C9, 15}, {3, 5, 3, C9, 16}};

struct Acc { double a[3][5]; };  // a[angle][l], l = 1..4
static Acc acceptance() {
  Acc A{};
  uint64_t st = 0x53507761766541ULL;  // fixed seed
  auto next = [&st]() {
    st += 0x9e3779b97f4a7c15ULL;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
  };
  for (int d = 0; d < 3; d++)
    for (int l = 1; l <= 4; l++) A.a[d][l] = -0.05 + 0.1 * (double(next() >> 11) * 0x1.0p-53);
  return A;
}
// eps factor of one angle as polynomial coefficients c0..c4 in x (Legendre P1..P4 expanded)
static std::vector<double> eps_poly(const Acc& A, int d) {
  const double* a = A.a[d];
  return {1.0 - 0.5 * a[2] + 0.375 * a[4], a[1] - 1.5 * a[3], 1.5 * a[2] - 3.75 * a[4], 2.5 * a[3], 4.375 * a[4]};
}
static double eps1(const std::vector<double>& c, double x) {
  return c[0] + x * (c[1] + x * (c[2] + x * (c[3] + x * c[4])));
}
// Gauss-Legendre nodes and weights on [-1, 1] (Newton iteration on P_n)
static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < n; i++) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; k++) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}
// I_k for every term
static std::vector<double> integrals(const Acc& A) {
  std::vector<double> gx, gw;
  gauss_legendre(256, gx, gw);
  const auto el = eps_poly(A, 0), ek = eps_poly(A, 1), ep = eps_poly(A, 2);
  auto cos_int = [&](const std::vector<double>& e, std::function<double(double)> f) {
    double s = 0.0;  // int_{-1}^{1} e(x) f(x) dx = int_0^pi e(cos t) f(cos t) sin t dt
    for (size_t i = 0; i < gx.size(); i++) {
      const double t = 0.5 * M_PI * (gx[i] + 1.0);
      s += gw[i] * 0.5 * M_PI * eps1(e, std::cos(t)) * f(std::cos(t)) * std::sin(t);
    }
    return s;
  };
  auto phi_int = [&](std::function<double(double)> f) {
    double s = 0.0;
    for (size_t i = 0; i < gx.size(); i++) {
      const double ph = M_PI * gx[i];
      s += gw[i] * M_PI * eps1(ep, gx[i]) * f(ph);
    }
    return s;
  };
  std::vector<double> I;
  for (const Term& t : TERMS)
    I.push_back(t.c * cos_int(el, [&](double x) { return fl(t.g, x); }) *
                cos_int(ek, [&](double x) { return fk(t.h, x); }) * phi_int([&](double x) { return fp(t.u, x); }));
  return I;
}

}  // namespace spw

template <typename kernelT, typename evalT>
class SPwaveAccPDF : public PDF<kernelT, evalT> {
 public:
  spw::Acc acc_;
  std::vector<double> I_;
  SPwaveAccPDF(dimension<evalT>* ctl, dimension<evalT>* ctk, dimension<evalT>* phi,
               const std::vector<parameter<evalT>*>& params) {
    this->dimensions_ = {ctl, ctk, phi};
    this->parameters_ = params;  // Fl S3 S4 S5 Afb S7 S8 S9 FS AS AS4 AS5 AS7 AS8
    acc_ = spw::acceptance();
    I_ = spw::integrals(acc_);
  }
  typedef std::unique_ptr<ComputeGraphNode<kernelT, evalT>> Ptr;
  std::string pn(int i) const { return this->parameters_.at(i)->get_name(); }
  Ptr coef(int k) const {
    constexpr auto V = &Variable<kernelT, evalT>;
    Ptr one_fs = 1.0 - V(pn(8));
    switch (k) {
      case 0: return one_fs->copy() * 3.0 / 4.0 * (1.0 - V(pn(0)));
      case 1: return one_fs->copy() * V(pn(0));
      case 2: return one_fs->copy() * 1.0 / 4.0 * (1.0 - V(pn(0)));
      case 3: return one_fs->copy() * (-V(pn(0)));
      case 7: return one_fs->copy() * 4.0 / 3.0 * V(pn(4));
      case 4: return one_fs->copy() * V(pn(1));
      case 5: return one_fs->copy() * V(pn(2));
      case 6: return one_fs->copy() * V(pn(3));
      case 8: return one_fs->copy() * V(pn(5));
      case 9: return one_fs->copy() * V(pn(6));
      case 10: return one_fs->copy() * V(pn(7));
      default: return V(pn(k - 11 + 8));  // FS, AS, AS4, AS5, AS7, AS8
    }
  }
  Ptr eps_graph(const std::string& var, double scale, int d) const {
    constexpr auto V = &Variable<kernelT, evalT>;
    const auto c = spw::eps_poly(acc_, d);
    Ptr x = scale == 1.0 ? V(var) : V(var) * scale;
    return c[0] + x->copy() * (c[1] + x->copy() * (c[2] + x->copy() * (c[3] + x->copy() * c[4])));
  }
  Ptr factor(int which, int i) const {
    constexpr auto V = &Variable<kernelT, evalT>;
    const std::string l = pn_dim(0), k = pn_dim(1), p = pn_dim(2);
    if (which == 0) {
      Ptr s = Sqrt<kernelT, evalT>(1.0 - V(l) * V(l));
      switch (i) { case 0: return Constant<kernelT, evalT>(1.0); case 1: return 2.0 * V(l) * V(l) - 1.0; case 2: return 1.0 - V(l) * V(l);
        case 3: return 2.0 * V(l) * std::move(s); case 4: return s; default: return V(l); }
    }
    if (which == 1) {
      Ptr s = Sqrt<kernelT, evalT>(1.0 - V(k) * V(k));
      switch (i) { case 0: return 1.0 - V(k) * V(k); case 1: return V(k) * V(k); case 2: return 2.0 * V(k) * std::move(s);
        case 3: return Constant<kernelT, evalT>(1.0); case 4: return V(k); default: return s; }
    }
    switch (i) { case 0: return Constant<kernelT, evalT>(1.0); case 1: return Cos<kernelT, evalT>(2.0 * V(p));
      case 2: return Cos<kernelT, evalT>(V(p)); case 3: return Sin<kernelT, evalT>(V(p)); default: return Sin<kernelT, evalT>(2.0 * V(p)); }
  }
  std::string pn_dim(int i) const { return this->dimensions_.at(i)->get_name(); }
  virtual Ptr prob() const override {
    Ptr eps = eps_graph(pn_dim(0), 1.0, 0) * eps_graph(pn_dim(1), 1.0, 1) * eps_graph(pn_dim(2), 1.0 / M_PI, 2);
    Ptr sum;
    for (int k = 0; k < 17; k++) {
      const spw::Term& t = spw::TERMS[k];
      Ptr ev = eps->copy() * (t.c * (factor(0, t.g) * factor(1, t.h) * factor(2, t.u)));
      Ptr term = coef(t.coef) * std::move(ev);
      sum = sum ? std::move(sum) + std::move(term) : std::move(term);
    }
    return sum;
  }
  virtual Ptr norm() const override {
    Ptr sum;
    for (int k = 0; k < 17; k++) {
      Ptr term = coef(spw::TERMS[k].coef) * I_[k];
      sum = sum ? std::move(sum) + std::move(term) : std::move(term);
    }
    return sum;
  }
  // density prob/norm at one point (double), for the generator bound
  double density(double ctl, double ctk, double phi) const {
    std::vector<double> th;
    for (auto* p : this->parameters_) th.push_back(p->get_value());
    auto cval = [&](int k) {
      const double ofs = 1.0 - th[8];
      switch (k) { case 0: return ofs * 0.75 * (1 - th[0]); case 1: return ofs * th[0]; case 2: return ofs * 0.25 * (1 - th[0]);
        case 3: return -ofs * th[0]; case 7: return ofs * 4.0 / 3.0 * th[4]; case 4: return ofs * th[1]; case 5: return ofs * th[2];
        case 6: return ofs * th[3]; case 8: return ofs * th[5]; case 9: return ofs * th[6]; case 10: return ofs * th[7];
        default: return th[k - 11 + 8]; }
    };
    const double e = spw::eps1(spw::eps_poly(acc_, 0), ctl) * spw::eps1(spw::eps_poly(acc_, 1), ctk) *
                     spw::eps1(spw::eps_poly(acc_, 2), phi / M_PI);
    double p = 0.0, nrm = 0.0;
    for (int k = 0; k < 17; k++) {
      const spw::Term& t = spw::TERMS[k];
      p += cval(t.coef) * e * t.c * spw::fl(t.g, ctl) * spw::fk(t.h, ctk) * spw::fp(t.u, phi);
      nrm += cval(t.coef) * I_[k];
    }
    return p / nrm;
  }
  // upper bound for accept-reject: 1.2 x the largest density on a 61^3 grid (ends included)
  virtual evalT get_max() const override {
    double m = 0.0;
    for (int i = 0; i <= 60; i++)
      for (int j = 0; j <= 60; j++)
        for (int k = 0; k <= 60; k++)
          m = std::max(m, density(-1.0 + i / 30.0, -1.0 + j / 30.0, M_PI * (-1.0 + k / 30.0)));
    return 1.2 * m;
  }
  double min_density() const {
    double m = 1e300;
    for (int i = 0; i <= 60; i++)
      for (int j = 0; j <= 60; j++)
        for (int k = 0; k <= 60; k++)
          m = std::min(m, density(-1.0 + i / 30.0, -1.0 + j / 30.0, M_PI * (-1.0 + k / 30.0)));
    return m;
  }
};

struct Workload {
  std::string name;
  std::vector<dimension<eT>*> dims;
  std::vector<parameter<eT>*> params;
  PDF<kT, eT>* pdf;
  bool optimize_dimensions;
  dimension<eT>* weight = nullptr;  // event weight column appended after generation
};

static Workload make_workload(const std::string& which) {
  Workload w;
  w.name = which;
  if (which == "mass" || which == "mass_w") {
    auto* m = new dimension<eT>("m", "m", 5000.0, 5600.0, false);
    auto* mb = new parameter<eT>("mb", "mb", 5280.0, 5200.0, 5400.0, 1.0, false);
    auto* sigma = new parameter<eT>("sigma", "sigma", 20.0, 5.0, 50.0, 0.5, false);
    auto* fsig = new parameter<eT>("fsig", "fsig", 0.3, 0.0, 1.0, 0.01, false);
    auto* alpha = new parameter<eT>("alpha", "alpha", -0.002, -0.01, 0.01, 0.0001, false);
    auto* gaus = new GaussianPDF<kT, eT>(m, mb, sigma);
    auto* ex = new ExponentialPDF<kT, eT>(m, alpha);
    w.pdf = new SumPDF<kT, eT>(gaus, ex, fsig);
    w.dims = {m};
    w.params = {mb, sigma, fsig, alpha};
    w.optimize_dimensions = false;
    if (which == "mass_w") w.weight = new dimension<eT>("w", "w", 0.0, 2.0, false);
  } else if (which == "cbpoly") {
    // Crystal Ball peak over a quadratic background on a normalised mass
    // x in [-1, 1]: conditionals, pow with a parameter exponent and the
    // polynomial's Horner form. The background 1 - 0.3 x + 0.1 x^2 falls
    // monotonically on the range, so PolynomialPDF::get_max's bound (range
    // limits only) holds.
    auto* x = new dimension<eT>("x", "x", -1.0, 1.0, false);
    auto* mu = new parameter<eT>("mu", "mu", 0.1, -0.2, 0.4, 0.001, false);
    auto* sigma = new parameter<eT>("sigma", "sigma", 0.05, 0.01, 0.2, 0.001, false);
    auto* alpha = new parameter<eT>("alpha", "alpha", 1.5, 0.5, 5.0, 0.01, false);
    auto* nn = new parameter<eT>("n", "n", 3.0, 1.5, 10.0, 0.05, false);
    auto* c1 = new parameter<eT>("c1", "c1", -0.3, -1.0, 1.0, 0.01, false);
    auto* c2 = new parameter<eT>("c2", "c2", 0.1, -1.0, 1.0, 0.01, false);
    auto* fsig = new parameter<eT>("fsig", "fsig", 0.3, 0.0, 1.0, 0.01, false);
    auto* cb = new CrystalballPDF<kT, eT>(x, mu, sigma, alpha, nn);
    auto* poly = new PolynomialPDF<kT, eT>(x, {c1, c2});
    w.pdf = new SumPDF<kT, eT>(cb, poly, fsig);
    w.dims = {x};
    w.params = {mu, sigma, alpha, nn, c1, c2, fsig};
    w.optimize_dimensions = false;
  } else if (which == "pwave") {
    auto* ctl = new dimension<eT>("ctl", "ctl", -1.0, 1.0, false);
    auto* ctk = new dimension<eT>("ctk", "ctk", -1.0, 1.0, false);
    auto* phi = new dimension<eT>("phi", "phi", -M_PI, +M_PI, false);
    auto* Fl = new parameter<eT>("Fl", "Fl", 0.70, 0.0, 1.0, 0.01, false);
    auto* S3 = new parameter<eT>("S3", "S3", -0.01, -1.0, 1.0, 0.01, false);
    auto* S4 = new parameter<eT>("S4", "S4", -0.15, -1.0, 1.0, 0.01, false);
    auto* S5 = new parameter<eT>("S5", "S5", -0.20, -1.0, 1.0, 0.01, false);
    auto* Afb = new parameter<eT>("Afb", "Afb", -0.10, -1.0, 1.0, 0.01, false);
    auto* S7 = new parameter<eT>("S7", "S7", 0.0, -1.0, 1.0, 0.01, false);
    auto* S8 = new parameter<eT>("S8", "S8", 0.0, -1.0, 1.0, 0.01, false);
    auto* S9 = new parameter<eT>("S9", "S9", 0.0, -1.0, 1.0, 0.01, false);
    w.pdf = new KstarmumuAngularPDF<kT, eT>(ctl, ctk, phi, Fl, S3, S4, S5, Afb, S7, S8, S9);
    w.dims = {ctl, ctk, phi};
    w.params = {Fl, S3, S4, S5, Afb, S7, S8, S9};
    w.optimize_dimensions = true;
  } else if (which == "spwave") {
    auto* ctl = new dimension<eT>("ctl", "ctl", -1.0, 1.0, false);
    auto* ctk = new dimension<eT>("ctk", "ctk", -1.0, 1.0, false);
    auto* phi = new dimension<eT>("phi", "phi", -M_PI, +M_PI, false);
    const char* names[14] = {"Fl", "S3", "S4", "S5", "Afb", "S7", "S8", "S9", "FS", "AS", "AS4", "AS5", "AS7", "AS8"};
    const double truth[14] = {0.70, -0.01, -0.15, -0.20, -0.10, 0.0, 0.0, 0.0, 0.05, -0.10, -0.03, 0.04, 0.02, -0.01};
    for (int i = 0; i < 14; i++)
      w.params.push_back(new parameter<eT>(names[i], names[i], truth[i], (i == 0 || i == 8) ? 0.0 : -1.0, 1.0, 0.01,
                                           false));
    auto* pdf = new SPwaveAccPDF<kT, eT>(ctl, ctk, phi, w.params);
    std::fprintf(stderr, "spwave: min density on the grid %.6g, generator bound %.6g\n", pdf->min_density(),
                 pdf->get_max());
    w.pdf = pdf;
    w.dims = {ctl, ctk, phi};
    w.optimize_dimensions = true;
  } else {
    std::fprintf(stderr, "unknown workload %s\n", which.c_str());
    std::exit(2);
  }
  return w;
}

static fitter_options make_fit_opts(const Workload& w) {
  fitter_options o;
  o.minimizer = fitter_options::minimizer_type::Minuit2;
  o.optimize_dimensions = w.optimize_dimensions;
  o.optimize_parameters = true;
  o.analytic_gradient = true;
  o.analytic_hessian = true;
  o.kahan_on_accelerator = true;
  o.print_level = 0;
  o.minuit_printlevel = 0;
  // Weighted data: the analytic Fisher kernel and the covariance correction
  // -2 H^-1 F H^-1 (fitter.hh:894-943; correct_weighted_fit defaults to true).
  o.analytic_fisher = w.weight != nullptr;
  o.correct_weighted_fit = true;
  return o;
}

static void generate(Workload& w, backendT* backend, Xoshiro128pp* rnd, unsigned n, EventVector<kT, eT>& out) {
  generator_options gen_opts;
  gen_opts.rndtype = generator_options::randomization_type::on_accelerator;
  gen_opts.print_level = 0;
  generator<kT, eT, backendT, blockT> gen(&gen_opts, backend, rnd);
  gen.generate(n, w.pdf, w.params, out);
  if (w.weight) {
    // Weights w_i = 0.5 + frac(i * 0.6180339887498949) in [0.5, 1.5), a
    // deterministic sequence uncorrelated with the generated events.
    out.add_dimensions({w.weight});
    const unsigned d = out.ndimensions() - 1;
    for (unsigned i = 0; i < n; i++) {
      double f = double(i) * 0.6180339887498949;
      f -= std::floor(f);
      out(i, d) = 0.5 + f;
    }
    out.set_event_weight(w.weight->get_name());
  }
}

// Parses "<prefix><name> = <expr>" lines printed by fitter::make_kernels at print_level 2.
static std::vector<std::pair<std::string, std::string>> grab(const std::string& log, const std::string& prefix) {
  std::vector<std::pair<std::string, std::string>> r;
  std::istringstream is(log);
  std::string line;
  while (std::getline(is, line)) {
    if (line.rfind(prefix, 0) != 0) continue;
    std::string rest = line.substr(prefix.size());
    size_t eq = rest.find(" = ");
    if (eq == std::string::npos) continue;
    r.push_back({rest.substr(0, eq), rest.substr(eq + 3)});
  }
  return r;
}
static std::string jpairs(const std::vector<std::pair<std::string, std::string>>& v) {
  std::string o = "[";
  for (size_t i = 0; i < v.size(); i++) o += (i ? "," : "") + ("[" + jstr(v[i].first) + "," + jstr(v[i].second) + "]");
  return o + "]";
}

static int cmd_golden(const std::string& which, unsigned n, const std::string& out_json, const std::string& out_bin) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  Workload w = make_workload(which);
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(229387429));
  EventVector<kT, eT> data(w.dims);
  recorded_kernels().clear();
  generate(w, &backend, &rnd, n, data);
  std::vector<RecordedKernel> gen_records = recorded_kernels();
  const uint64_t ev_hash = fnv1a(data.get_data(), data.buffer_size());
  if (!out_bin.empty()) {
    FILE* f = std::fopen(out_bin.c_str(), "wb");
    std::fwrite(data.get_data(), 1, data.buffer_size(), f);
    std::fclose(f);
  }
  std::vector<double> truth;
  for (auto* p : w.params) truth.push_back(p->get_value());

  fitter_options fopts = make_fit_opts(w);
  fopts.print_level = 2;  // make_kernels prints the hoisted buffer expressions
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  recorded_kernels().clear();
  // fit() runs make_kernels once (a second make_kernels on one fitter would
  // re-grow its result dimension vectors, fitter.hh:544).
  std::ostringstream captured;
  auto* old = std::cout.rdbuf(captured.rdbuf());
  auto t0 = std::chrono::steady_clock::now();
  fit.fit(w.pdf, w.params, &data);
  auto t1 = std::chrono::steady_clock::now();
  std::cout.rdbuf(old);
  fopts.print_level = 0;
  std::string log = captured.str();
  std::vector<double> values, errors;
  for (auto* p : w.params) {
    values.push_back(p->get_value());
    errors.push_back(p->get_error());
  }
  const int npar = int(w.params.size());

  // Evaluation points: truth, fitted minimum, and a displaced point.
  std::vector<std::vector<double>> points = {truth, values};
  {
    std::vector<double> d = truth;
    // half an error from the truth, alternating in sign, kept within each
    // parameter's limits (a poorly constrained parameter would leave them)
    for (int i = 0; i < npar; i++)
      d[i] = std::min(std::max(truth[i] + 0.5 * errors[i] * ((i % 2) ? -1.0 : 1.0), w.params[i]->get_min()),
                      w.params[i]->get_max());
    points.push_back(d);
  }
  std::string pts = "[";
  for (size_t k = 0; k < points.size(); k++) {
    for (int i = 0; i < npar; i++) w.params[i]->set_value(points[k][i]);
    Capture cap;
    g_capture = &cap;
    std::cout.rdbuf(captured.rdbuf());
    double nll = fit.likelihood();
    std::vector<double> grad(npar);
    double nll2 = fit.likelihood_and_gradient(npar, grad.data());
    std::vector<double> h(npar * npar);
    fit.hessian(npar, h.data());
    std::vector<double> fm;
    if (w.weight) {
      fm.resize(size_t(npar) * npar);
      fit.fisher(w.pdf, w.params, &data, npar, fm.data());
    }
    std::cout.rdbuf(old);
    g_capture = nullptr;
    pts += std::string(k ? "," : "") + "{\"params\":" + jvec(points[k]) + ",\"nll\":" + jnum(nll) +
           ",\"nll_from_grad_kernel\":" + jnum(nll2) + ",\"grad\":" + jvec(grad) + ",\"hessian\":" + jvec(h) +
           (w.weight ? ",\"fisher\":" + jvec(fm) : std::string()) + ",\"kernel_params\":{";
    bool first = true;
    for (auto& kv : cap.params) {
      pts += std::string(first ? "" : ",") + jstr(kv.first) + ":" + jvec(kv.second);
      first = false;
    }
    pts += "},\"kernel_sums\":{";
    first = true;
    for (auto& kv : cap.sums) {
      pts += std::string(first ? "" : ",") + jstr(kv.first) + ":" + jvec(kv.second);
      first = false;
    }
    pts += "}}";
  }
  pts += "]";

  std::string kern = "[";
  std::vector<RecordedKernel> all = gen_records;
  for (auto& r : recorded_kernels()) all.push_back(r);
  for (size_t i = 0; i < all.size(); i++) {
    auto& r = all[i];
    kern += std::string(i ? "," : "") + "{\"name\":" + jstr(r.name) + ",\"inputs\":" + jsvec(r.inputs) +
            ",\"outputs\":" + jsvec(r.outputs) + ",\"params\":" + jsvec(r.params) + ",\"exprs\":" + jsvec(r.exprs) +
            ",\"kahan\":" + (r.kahan ? "true" : "false");
    if (r.generate)
      kern += ",\"generate\":true,\"lo\":" + jvec(r.lo) + ",\"hi\":" + jvec(r.hi) + ",\"maxprob\":" + jnum(r.maxprob);
    kern += "}";
  }
  kern += "]";
  std::vector<std::string> dnames, pnames;
  for (auto* d : w.dims) dnames.push_back(d->get_name());
  if (w.weight) dnames.push_back(w.weight->get_name());
  for (auto* p : w.params) pnames.push_back(p->get_name());
  char hash[32];
  std::snprintf(hash, sizeof hash, "%016llx", (unsigned long long)ev_hash);
  std::string js = "{\"workload\":" + jstr(w.name) + ",\"nevents\":" + std::to_string(n) +
                   ",\"seed\":229387429,\"events_fnv1a\":" + jstr(hash) + ",\"dimensions\":" + jsvec(dnames) +
                   ",\"parameters\":" + jsvec(pnames) + ",\"truth\":" + jvec(truth) +
                   ",\"maxprob\":" + jnum(w.pdf->get_max()) + ",\"kernels\":" + kern +
                   ",\"event_buffers\":" + jpairs(grab(log, "EVENTBUFFER ")) +
                   ",\"lh_buffers\":" + jpairs(grab(log, "BUFFER ")) +
                   ",\"grad_buffers\":" + jpairs(grab(log, "GRADBUFFER: ")) +
                   ",\"hessian_buffers\":" + jpairs(grab(log, "HESSIANBUFFER: ")) +
                   (w.weight ? ",\"weight\":" + jstr(w.weight->get_name()) +
                                   ",\"fisher_buffers\":" + jpairs(grab(log, "FISHERBUFFER: "))
                             : std::string()) +
                   ",\"fit\":{\"values\":" +
                   jvec(values) + ",\"errors\":" + jvec(errors) + ",\"wall_ms\":" +
                   jnum(std::chrono::duration<double, std::milli>(t1 - t0).count()) + "},\"points\":" + pts + "}\n";
  FILE* f = std::fopen(out_json.c_str(), "w");
  std::fputs(js.c_str(), f);
  std::fclose(f);
  std::fprintf(stderr, "golden %s n=%u events_fnv1a=%s fit_ms=%.1f\n", which.c_str(), n, hash,
               std::chrono::duration<double, std::milli>(t1 - t0).count());
  return 0;
}

// Times NLL+gradient evaluations of the reference kernel text at nthreads.
static int cmd_bench(const std::string& which, unsigned n, unsigned nthreads, unsigned nevals) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  Workload w = make_workload(which);
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(229387429));
  EventVector<kT, eT> data(w.dims);
  generate(w, &backend, &rnd, n, data);
  copts.llvm_nthreads = nthreads;
  fitter_options fopts = make_fit_opts(w);
  fopts.minuit_maxcalls = 1;
  fopts.minuit_maxiterations = 1;
  fopts.postrun_hesse = false;
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  std::ostringstream sink;
  auto* old = std::cout.rdbuf(sink.rdbuf());
  fit.fit(w.pdf, w.params, &data);
  const int npar = int(w.params.size());
  std::vector<double> grad(npar);
  for (int i = 0; i < 3; i++) fit.likelihood_and_gradient(npar, grad.data());
  auto t0 = std::chrono::steady_clock::now();
  double acc = 0;
  for (unsigned i = 0; i < nevals; i++) acc += fit.likelihood_and_gradient(npar, grad.data());
  auto t1 = std::chrono::steady_clock::now();
  std::cout.rdbuf(old);
  double s = std::chrono::duration<double>(t1 - t0).count();
  std::printf("{\"workload\":\"%s\",\"nevents\":%u,\"nthreads\":%u,\"nevals\":%u,\"evals_per_s\":%.6g,\"nll\":%.17g}\n",
              which.c_str(), n, nthreads, nevals, nevals / s, acc / nevals);
  return 0;
}

// Toy study with the reference's own generator and fitter, one toy at a
// time as toystudy::toy does (toystudy.hh:55-82), except that every toy's
// truth is the workload's truth times (1 + u), u uniform in [-jitter, jitter]
// (SplitMix64 stream), and the event count is the reference's
// RandomGenerator::poisson(mean) (random.hh:42-80) clipped to [200, 50000].
// Each toy is generated at its truth (the generate kernel is rebuilt per toy
// because the generator substitutes the parameter values into it,
// generator.hh:145) and fitted from it (MIGRAD + HESSE). Writes the pulls.
static int cmd_toys(const std::string& which, unsigned ntoys, double mean, double jitter, const std::string& out,
                    uint64_t seed = 229387429) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  Workload w = make_workload(which);
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(seed));
  generator_options gen_opts;
  gen_opts.rndtype = generator_options::randomization_type::on_accelerator;
  gen_opts.print_level = 0;
  generator<kT, eT, backendT, blockT> gen(&gen_opts, &backend, &rnd);
  fitter_options fopts = make_fit_opts(w);
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  std::vector<double> base;
  for (auto* p : w.params) base.push_back(p->get_value());
  uint64_t sm = 0x746f79737475ULL + (seed - 229387429);
  auto uni = [&sm]() {
    sm += 0x9e3779b97f4a7c15ULL;
    uint64_t z = sm;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return double((z ^ (z >> 31)) >> 11) * 0x1.0p-53;
  };
  std::string pulls = "[", truths = "[", counts = "[";
  unsigned nconv = 0;
  std::ostringstream sink;
  auto* old = std::cout.rdbuf(sink.rdbuf());
  for (unsigned t = 0; t < ntoys; t++) {
    std::vector<double> truth(base.size());
    for (size_t i = 0; i < base.size(); i++) truth[i] = base[i] * (1.0 + jitter * (2.0 * uni() - 1.0));
    for (size_t i = 0; i < base.size(); i++) {
      w.params[i]->set_value(truth[i]);
      w.params[i]->set_start_value(truth[i]);
    }
    unsigned n = rnd.poisson(mean);
    n = std::min(50000u, std::max(200u, n));
    EventVector<kT, eT> data(w.dims, n);
    gen.generate(n, w.pdf, w.params, data, false);
    for (size_t i = 0; i < base.size(); i++) w.params[i]->set_value(truth[i]);
    const bool ok = fit.fit(w.pdf, w.params, &data, t > 0);
    nconv += ok ? 1 : 0;
    std::vector<double> pl;
    for (size_t i = 0; i < base.size(); i++)
      pl.push_back((w.params[i]->get_value() - truth[i]) / w.params[i]->get_error());
    pulls += std::string(t ? "," : "") + jvec(pl);
    truths += std::string(t ? "," : "") + jvec(truth);
    counts += std::string(t ? "," : "") + std::to_string(n);
  }
  std::cout.rdbuf(old);
  std::string js = "{\"workload\":" + jstr(which) + ",\"ntoys\":" + std::to_string(ntoys) + ",\"mean\":" + jnum(mean) +
                   ",\"jitter\":" + jnum(jitter) + ",\"converged\":" + std::to_string(nconv) + ",\"counts\":" +
                   counts + "],\"truths\":" + truths + "],\"pulls\":" + pulls + "]}\n";
  FILE* f = std::fopen(out.c_str(), "w");
  std::fputs(js.c_str(), f);
  std::fclose(f);
  std::fprintf(stderr, "toys %s: %u of %u fits converged\n", which.c_str(), nconv, ntoys);
  return 0;
}

// Runs the reference's plotter (matplotlib output, pulls on) on generated
// events at the truth and records: the integral kernel it builds (parameter
// values substituted, plotter.hh:138-216) with its per-bin integrals, the
// written .py text, and the same definite integral with the parameters kept
// as names (parameter-only terms hoisted into buffers as the fitter does),
// for a backend that takes parameter values at launch.
static int cmd_plot(const std::string& which, unsigned n, const std::string& var, unsigned nbins,
                    const std::string& out_py, const std::string& out_json) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  Workload w = make_workload(which);
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(229387429));
  EventVector<kT, eT> data(w.dims);
  generate(w, &backend, &rnd, n, data);
  const uint64_t ev_hash = fnv1a(data.get_data(), data.buffer_size());

  plotter_options popts;
  popts.plotter = plotter_options::plotter_type::MatPlotLib;
  popts.plot_pulls = true;
  popts.print_level = 0;
  plotter<kT, eT, backendT, blockT> pl(&popts, &backend);
  recorded_kernels().clear();
  Capture cap;
  g_capture = &cap;
  std::ostringstream captured;
  auto* old = std::cout.rdbuf(captured.rdbuf());
  pl.plot(w.pdf, w.params, &data, var, out_py, "", nbins);
  // the same plot as a ROOT macro (same stem, kernels reused)
  const std::string out_c = out_py.substr(0, out_py.size() - 3) + ".C";
  popts.plotter = plotter_options::plotter_type::Root;
  pl.plot(w.pdf, w.params, &data, var, out_c, "", nbins, 0.0, 0.0, true);
  std::cout.rdbuf(old);
  g_capture = nullptr;
  RecordedKernel rk;
  for (auto& r : recorded_kernels())
    if (r.name == "integral_kernel") rk = r;
  std::vector<double> pdf_y = cap.outputs["integral_kernel"];
  pdf_y.resize(size_t(nbins) * popts.pdf_bin_multiplier);

  // the integral with symbolic parameters (plotter::make_kernels without the
  // parameter substitution)
  std::vector<std::string> dn, floating;
  std::vector<eT> dv;
  std::string vfrom, vto;
  double lo = 0.0, hi = 0.0;
  for (auto* d : w.pdf->dimensions())
    if (d->get_name() != var) {
      dn.push_back(d->get_from_name());
      dv.push_back(d->get_min());
      dn.push_back(d->get_to_name());
      dv.push_back(d->get_max());
    } else {
      vfrom = d->get_from_name();
      vto = d->get_to_name();
      lo = d->get_min();
      hi = d->get_max();
    }
  for (auto* p : w.params) floating.push_back(p->get_name());
  std::unique_ptr<ComputeGraphNode<kT, eT>> integral = w.pdf->definite_integral()->substitute(dn, dv)->simplify();
  integral->rename_variable(vfrom, "morefit_from");
  integral->rename_variable(vto, "morefit_to");
  std::vector<std::string> bnames;
  std::vector<std::unique_ptr<ComputeGraphNode<kT, eT>>> bexprs;
  std::unique_ptr<ComputeGraphNode<kT, eT>> sym =
      integral->optimize_buffering_constant_terms(bnames, bexprs, floating, "morefit_parambuffer_", 2.0);
  std::vector<std::pair<std::string, std::string>> bufs;
  for (size_t i = 0; i < bnames.size(); i++) bufs.push_back({bnames[i], bexprs[i]->get_kernel()});
  std::vector<std::string> sparams = floating;
  for (auto& b : bnames) sparams.push_back(b);

  std::ifstream pyf(out_py), cf(out_c);
  std::stringstream pys, cs;
  pys << pyf.rdbuf();
  cs << cf.rdbuf();
  std::vector<std::string> tex;
  for (auto* d : w.pdf->dimensions()) tex.push_back(d->get_tex());
  std::vector<double> truth;
  for (auto* p : w.params) truth.push_back(p->get_value());
  char hash[32];
  std::snprintf(hash, sizeof hash, "%016llx", (unsigned long long)ev_hash);
  std::string js = "{\"workload\":" + jstr(w.name) + ",\"nevents\":" + std::to_string(n) +
                   ",\"events_fnv1a\":" + jstr(hash) + ",\"variable\":" + jstr(var) +
                   ",\"nbins\":" + std::to_string(nbins) +
                   ",\"pdf_bin_multiplier\":" + std::to_string(popts.pdf_bin_multiplier) +
                   ",\"range\":" + jvec({lo, hi}) + ",\"parameters\":" + jsvec(floating) +
                   ",\"truth\":" + jvec(truth) + ",\"reference_kernel\":{\"inputs\":" + jsvec(rk.inputs) +
                   ",\"params\":" + jsvec(rk.params) + ",\"exprs\":" + jsvec(rk.exprs) +
                   "},\"pdf_y\":" + jvec(pdf_y) + ",\"integral\":{\"inputs\":" +
                   jsvec({"morefit_from", "morefit_to"}) + ",\"params\":" + jsvec(sparams) +
                   ",\"exprs\":" + jsvec({sym->get_kernel()}) + ",\"buffers\":" + jpairs(bufs) +
                   "},\"tex\":" + jsvec(tex) + ",\"py\":" + jstr(pys.str()) + ",\"C\":" + jstr(cs.str()) +
                   "}\n";
  FILE* f = std::fopen(out_json.c_str(), "w");
  std::fputs(js.c_str(), f);
  std::fclose(f);
  std::fprintf(stderr, "plot %s %s n=%u bins=%u events_fnv1a=%s\n", which.c_str(), var.c_str(), n, nbins, hash);
  return 0;
}

// Fits datasets from a file with the reference's fitter: the file holds, per
// dataset, uint32 n, npar doubles (truth, also the start point) and the SoA
// events (ndims x n doubles). Writes values and errors per dataset.
static int cmd_fitfile(const std::string& which, const std::string& in, const std::string& out) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  Workload w = make_workload(which);
  fitter_options fopts = make_fit_opts(w);
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  FILE* f = std::fopen(in.c_str(), "rb");
  if (!f) return 2;
  const size_t npar = w.params.size(), nd = w.dims.size();
  std::string vals = "[", errs = "[";
  std::ostringstream sink;
  auto* old = std::cout.rdbuf(sink.rdbuf());
  for (unsigned t = 0;; t++) {
    uint32_t n = 0;
    if (std::fread(&n, 4, 1, f) != 1) break;
    std::vector<double> truth(npar);
    if (std::fread(truth.data(), 8, npar, f) != npar) break;
    EventVector<kT, eT> data(w.dims, n);
    if (std::fread(data.get_data(), 8, nd * n, f) != nd * n) break;
    for (size_t i = 0; i < npar; i++) {
      w.params[i]->set_value(truth[i]);
      w.params[i]->set_start_value(truth[i]);
    }
    fit.fit(w.pdf, w.params, &data, t > 0);
    std::vector<double> v, e;
    for (auto* p : w.params) {
      v.push_back(p->get_value());
      e.push_back(p->get_error());
    }
    vals += std::string(t ? "," : "") + jvec(v);
    errs += std::string(t ? "," : "") + jvec(e);
  }
  std::cout.rdbuf(old);
  std::fclose(f);
  FILE* o = std::fopen(out.c_str(), "w");
  std::fputs(("{\"values\":" + vals + "],\"errors\":" + errs + "]}\n").c_str(), o);
  std::fclose(o);
  return 0;
}

int main(int argc, char** argv) {
  install_capture();
  if (argc >= 5 && std::string(argv[1]) == "fitfile") return cmd_fitfile(argv[2], argv[3], argv[4]);
  if (argc >= 5 && std::string(argv[1]) == "golden")
    return cmd_golden(argv[2], unsigned(std::stoul(argv[3])), argv[4], argc > 5 ? argv[5] : "");
  if (argc >= 6 && std::string(argv[1]) == "bench")
    return cmd_bench(argv[2], unsigned(std::stoul(argv[3])), unsigned(std::stoul(argv[4])),
                     unsigned(std::stoul(argv[5])));
  if (argc >= 8 && std::string(argv[1]) == "plot")
    return cmd_plot(argv[2], unsigned(std::stoul(argv[3])), argv[4], unsigned(std::stoul(argv[5])), argv[6], argv[7]);
  if (argc >= 7 && std::string(argv[1]) == "toys")
    return cmd_toys(argv[2], unsigned(std::stoul(argv[3])), std::stod(argv[4]), std::stod(argv[5]), argv[6],
                    argc > 7 ? std::stoull(argv[7]) : 229387429ULL);
  std::fprintf(stderr, "usage: refkit golden <mass|mass_w|cbpoly|pwave|spwave> <n> <out.json> [events.bin]\n"
                       "       refkit bench <mass|pwave|spwave> <n> <nthreads> <nevals>\n"
                       "       refkit toys <pwave> <ntoys> <mean events> <jitter> <out.json> [seed]\n"
                       "       refkit plot <workload> <n> <variable> <nbins> <out.py> <out.json>\n"
                       "       refkit fitfile <workload> <datasets.bin> <out.json>\n");
  return 2;
}
