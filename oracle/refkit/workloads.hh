// Workload definitions shared by the oracle kit (refkit.cc) and the C++
// drop-in test (tests/cpp/dropin.cc): the models, parameters, ranges and
// fitter options of the golden vectors, templated on the reference's
// kernelT/evalT so the drop-in can build them in FP64 and in mixed precision.
//
// TEST INFRASTRUCTURE ONLY: compiled together with the reference's own
// headers (graph.hh, pdf.hh, physicspdfs.hh, fitter.hh); nothing in the
// product includes it. Include after fitter.hh.
#ifndef MOREFIT_ORACLE_WORKLOADS_HH
#define MOREFIT_ORACLE_WORKLOADS_HH

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <string>
#include <vector>

namespace morefit {


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

template <typename kT, typename eT>
struct Workload {
  std::string name;
  std::vector<dimension<eT>*> dims;
  std::vector<parameter<eT>*> params;
  PDF<kT, eT>* pdf;
  bool optimize_dimensions;
  dimension<eT>* weight = nullptr;  // event weight column appended after generation
};

template <typename kT, typename eT>
Workload<kT, eT> make_workload(const std::string& which) {
  Workload<kT, eT> w;
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

template <typename kT, typename eT>
fitter_options make_fit_opts(const Workload<kT, eT>& w) {
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

}  // namespace morefit

#endif
