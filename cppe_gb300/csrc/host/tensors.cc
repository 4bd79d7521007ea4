// Cartesian interaction tensors T_k(R) = d^k phi(|R|) / dR^k of the Coulomb
// potential phi = 1/R and of the Thole-damped potential
// phi = (1 - (1 + v/2) e^-v) / R, v = a R -- the reference's tensors
// submodule (src/python_iface/export_tensors.cc:17-40 over
// src/core/tensors/tensors_autogen.cc and tensors_recursive.cc), used by
// callers that assemble dense operators or check fields by hand.  These are
// host utilities off the solve path: the GPU kernels evaluate the same
// tensors inline.
//
// Method (our own): a radial function depends on x, y, z only through
// s = R^2 / 2, so with F(s) = phi and d/ds = (1/R) d/dR,
//   d^nx/dx d^ny/dy d^nz/dz F = sum_{i,j,l} h(nx,i) h(ny,j) h(nz,l)
//                                x^(2i-nx) y^(2j-ny) z^(2l-nz) F^(i+j+l)(s),
//   h(n,i) = n! / ((2i-n)! (n-i)! 2^(n-i)),  ceil(n/2) <= i <= n,
// and the radial derivatives g_m = ((1/R) d/dR)^m phi are exact:
//   ((1/R) d/dR)^m R^-1 = (-1)^m (2m-1)!! R^-(2m+1),
//   (1/R) d/dR [R^p e^-aR] = (p R^(p-2) - a R^(p-1)) e^-aR.
// Components are ordered as the reference's xyz2idx (x, then y, descending).
#include <cmath>
#include <map>
#include <stdexcept>

#include "cppe_host.hh"

namespace libcppe {
namespace {

double fact(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f *= i;
  return f;
}

// h(n, i) of the one-coordinate derivative of F(x^2/2 + c)
double hcoef(int n, int i) {
  if (2 * i < n || i > n) return 0.0;
  return fact(n) / (fact(2 * i - n) * fact(n - i) * std::ldexp(1.0, n - i));
}

// g_m = ((1/R) d/dR)^m phi for m = 0..k, undamped (a = 0) or Thole-damped
std::vector<double> radial_derivatives(int k, double R, double a) {
  std::vector<double> g(k + 1, 0.0);
  // Coulomb part
  double dfac = 1.0;  // (2m-1)!!
  for (int m = 0; m <= k; ++m) {
    if (m > 0) dfac *= (2 * m - 1);
    g[m] = ((m & 1) ? -dfac : dfac) * std::pow(R, -(2 * m + 1));
  }
  if (a != 0.0) {
    // exponential part: sum_p c_p R^p e^-aR, starting from -(R^-1 + a/2) e^-aR
    std::map<int, double> c{{-1, -1.0}, {0, -0.5 * a}};
    const double e = std::exp(-a * R);
    for (int m = 0; m <= k; ++m) {
      double s = 0.0;
      for (const auto& t : c) s += t.second * std::pow(R, t.first);
      g[m] += s * e;
      std::map<int, double> nc;
      for (const auto& t : c) {
        if (t.first != 0) nc[t.first - 2] += t.first * t.second;
        nc[t.first - 1] -= a * t.second;
      }
      c.swap(nc);
    }
  }
  return g;
}

Vector cartesian_tensor(int k, const std::array<double, 3>& R, double a) {
  if (k < 0) throw std::invalid_argument("tensor order must be non-negative");
  const double r = std::sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  const std::vector<double> g = radial_derivatives(k, r, a);
  Vector out;
  out.reserve(multipole_components(k));
  for (int x = k; x >= 0; --x)
    for (int y = k - x; y >= 0; --y) {
      const int z = k - x - y;
      double t = 0.0;
      for (int i = (x + 1) / 2; i <= x; ++i)
        for (int j = (y + 1) / 2; j <= y; ++j)
          for (int l = (z + 1) / 2; l <= z; ++l)
            t += hcoef(x, i) * hcoef(y, j) * hcoef(z, l) * std::pow(R[0], 2 * i - x) *
                 std::pow(R[1], 2 * j - y) * std::pow(R[2], 2 * l - z) * g[i + j + l];
      out.push_back(t);
    }
  return out;
}

}  // namespace

Vector T_tensor(int k, const std::array<double, 3>& R) { return cartesian_tensor(k, R, 0.0); }

Vector T_tensor_damp_thole(int k, const std::array<double, 3>& R, double a) {
  return cartesian_tensor(k, R, a);
}

// T_recursive (tensors_recursive.cc:6-21): the damping argument is the Thole
// a of the pair (v = a R); damped tensors above third order are refused there
// ("Thole damping only implemented up to third order.").
Vector T_recursive(int k, const std::array<double, 3>& R, double damping_factor) {
  if (damping_factor != 0.0 && k > 3)
    throw std::runtime_error("Thole damping only implemented up to third order.");
  return cartesian_tensor(k, R, damping_factor);
}

// position of (x, y, z) among the components of order x + y + z
// (tensors_recursive.cc:24-42); -1 for negative arguments
int xyz2idx(int x, int y, int z) {
  if (x < 0 || y < 0 || z < 0) return -1;
  const int k = x + y + z;
  int idx = 0;
  for (int a = k; a > x; --a) idx += k - a + 1;  // components with a larger x power
  return idx + (k - x - y);                      // then y descending
}

}  // namespace libcppe
