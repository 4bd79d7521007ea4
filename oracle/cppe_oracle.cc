// Test infrastructure (oracle) -- never linked into the product.
//
// A CPU restatement of the reference's induced-dipole hot path, used by the
// tests as the parity checker and by bench.py as the timed CPU baseline.  It
// follows the reference algorithm step by step, in code of its own:
//
//   octree build           src/core/fmm/tree.cc:134-237, add_child :94-109,
//                          split_cell :111-132, Cell::Cell :11-24
//   interaction lists      interact_dehnen_lazy   src/core/fmm/calculate.cc:74-127
//   FMM passes             evaluate_P2M :129-157, evaluate_M2M :159-184,
//                          evaluate_M2L_lazy :186-203, evaluate_P2P_lazy :205-225,
//                          evaluate_L2L :227-243, evaluate_L2P :245-260,
//                          Tree::compute_field_fmm tree.cc:359-385
//   direct sums            evaluate_direct{,_damping} calculate.cc:262-300
//   pair kernels           P2P<m,3> (plain and Thole-damped), field_m{0,1,2}.cc;
//                          here written in closed form from the derivatives of
//                          the damped potential f_v(aR)/R with the screening
//                          factors of tensors_recursive.cc:93-114
//   Cartesian operators    M2M/M2L/L2L/L2P of field_m{0,1,2}.cc (Dehnen
//                          convention, fmmgen index order; sizes utils.cc:3-20),
//                          here evaluated from index tables for any order
//   MultipoleFields        src/core/electric_fields.cc:106-189
//   BMatrix::apply         src/core/bmatrix.cc:9-40, diagonal ops :42-62
//   InducedMoments (PCG)   src/core/electric_fields.cc:191-239
//
// Parity is pinned by tests against the reference's golden vectors and, where
// the reference sources are mounted, against the reference compiled in place.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace orc {

constexpr int PMAX = 9;

constexpr int nterms(int p) { return p < 0 ? 0 : (p + 1) * (p + 2) * (p + 3) / 6; }

// Multi-indices ordered by total order, then x descending, then y descending
// (the order of xyz2idx, tensors_recursive.cc:24-39, and of fmmgen's arrays).
struct Index {
  int nx[nterms(PMAX)], ny[nterms(PMAX)], nz[nterms(PMAX)];
  int ix[PMAX + 1][PMAX + 1][PMAX + 1];
  Index() {
    int j = 0;
    for (int o = 0; o <= PMAX; ++o)
      for (int a = o; a >= 0; --a)
        for (int b = o - a; b >= 0; --b) {
          int c = o - a - b;
          nx[j] = a, ny[j] = b, nz[j] = c;
          ix[a][b][c] = j++;
        }
  }
  int at(int a, int b, int c) const { return ix[a][b][c]; }
};
const Index& IDX() {
  static Index I;
  return I;
}

struct Term {
  int out, in, w;  // out += weight[w] * in
};

// Operator term tables for source order m and expansion order p.
struct Ops {
  int m, p, msize, lsize, moff;
  std::vector<Term> m2m;  // Ms[out] += mono[w] * M[in]
  std::vector<Term> m2l;  // L[out]  += D[w]    * M[in]
  std::vector<Term> l2l;  // Ls[out] += mono[w] * L[in]
  std::vector<Term> l2p;  // F[out]  -= mono[w] * L[in]
  std::vector<Term> p2m;  // M[out]  += mono[w] * S[in]
};

const Ops& ops(int m, int p) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, Ops> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_pair(m, p);
  auto it  = cache.find(key);
  if (it != cache.end()) return it->second;
  const Index& I = IDX();
  Ops o;
  o.m     = m;
  o.p     = p;
  o.moff  = nterms(m - 1);
  o.msize = nterms(p) - o.moff;
  o.lsize = nterms(p - m);
  // M2M: n, k with m <= |k| <= |n| <= p and k <= n componentwise.
  for (int n = o.moff; n < nterms(p); ++n)
    for (int k = o.moff; k <= n; ++k) {
      int dx = I.nx[n] - I.nx[k], dy = I.ny[n] - I.ny[k], dz = I.nz[n] - I.nz[k];
      if (dx < 0 || dy < 0 || dz < 0) continue;
      o.m2m.push_back({n - o.moff, k - o.moff, I.at(dx, dy, dz)});
    }
  // P2M: the same with only |k| == m source terms.
  for (const Term& t : o.m2m)
    if (t.in < nterms(m) - o.moff) o.p2m.push_back(t);
  // M2L: |n| <= p - m, m <= |k|, |n| + |k| <= p; weight D_{n+k}.
  for (int n = 0; n < o.lsize; ++n) {
    int on = I.nx[n] + I.ny[n] + I.nz[n];
    for (int k = o.moff; k < nterms(p - on); ++k)
      o.m2l.push_back({n, k - o.moff, I.at(I.nx[n] + I.nx[k], I.ny[n] + I.ny[k],
                                           I.nz[n] + I.nz[k])});
  }
  // L2L: Ls_n += sum_{k >= n} d^{k-n}/(k-n)! L_k.
  for (int n = 0; n < o.lsize; ++n)
    for (int k = n; k < o.lsize; ++k) {
      int dx = I.nx[k] - I.nx[n], dy = I.ny[k] - I.ny[n], dz = I.nz[k] - I.nz[n];
      if (dx < 0 || dy < 0 || dz < 0) continue;
      o.l2l.push_back({n, k, I.at(dx, dy, dz)});
    }
  // L2P: F_c -= sum_{n >= e_c} t^{n-e_c}/(n-e_c)! L_n.
  for (int c = 0; c < 3; ++c)
    for (int n = 1; n < o.lsize; ++n) {
      int d[3] = {I.nx[n], I.ny[n], I.nz[n]};
      if (d[c] == 0) continue;
      d[c] -= 1;
      o.l2p.push_back({c, n, I.at(d[0], d[1], d[2])});
    }
  return cache.emplace(key, std::move(o)).first->second;
}

// mono[j] = d^j / j! for |j| <= p.
void monomials(double dx, double dy, double dz, int p, double* mono) {
  const Index& I = IDX();
  double px[PMAX + 1], py[PMAX + 1], pz[PMAX + 1];
  px[0] = py[0] = pz[0] = 1.0;
  for (int a = 1; a <= p; ++a) {
    px[a] = px[a - 1] * dx / a;
    py[a] = py[a - 1] * dy / a;
    pz[a] = pz[a - 1] * dz / a;
  }
  for (int j = 0; j < nterms(p); ++j) mono[j] = px[I.nx[j]] * py[I.ny[j]] * pz[I.nz[j]];
}

// D[j] = d^j (1/R) for |j| <= p by the recurrence
//   |n| R^2 D_n = -(2|n|-1) sum_i n_i r_i D_{n-e_i} - (|n|-1) sum_i n_i(n_i-1) D_{n-2e_i}
// (obtained by differentiating R^2 d_i(1/R) = -r_i / R).
void derivs(double x, double y, double z, int p, double* D) {
  const Index& I = IDX();
  double r2      = x * x + y * y + z * z;
  double ir2     = 1.0 / r2;
  D[0]           = std::sqrt(ir2);
  double r[3]    = {x, y, z};
  for (int j = 1; j < nterms(p); ++j) {
    int n[3] = {I.nx[j], I.ny[j], I.nz[j]};
    int o    = n[0] + n[1] + n[2];
    double s = 0.0, t = 0.0;
    for (int i = 0; i < 3; ++i) {
      if (n[i] >= 1) {
        int q[3] = {n[0], n[1], n[2]};
        q[i] -= 1;
        s += n[i] * r[i] * D[I.at(q[0], q[1], q[2])];
      }
      if (n[i] >= 2) {
        int q[3] = {n[0], n[1], n[2]};
        q[i] -= 2;
        t += n[i] * (n[i] - 1) * D[I.at(q[0], q[1], q[2])];
      }
    }
    D[j] = -((2 * o - 1) * s + (o - 1) * t) * ir2 / o;
  }
}

// Thole screening of the radial derivative factors G_q(R) = (R^-1 d/dR)^q g,
// g = f_v(aR)/R: G_1 = -f_E/R^3, G_2 = 3 f_T/R^5, G_3 = -15 f_D/R^7.
inline void radial(double R, double a, double* G) {
  double iR = 1.0 / R, iR2 = iR * iR;
  double iR3 = iR * iR2;
  double fE = 1.0, fT = 1.0, fD = 1.0;
  if (a > 0.0) {
    double v  = a * R;
    double e  = std::exp(-v);
    double fv = 1.0 - (0.5 * v + 1.0) * e;
    fE        = fv - (0.5 * v * v + 0.5 * v) * e;
    fT        = fE - v * v * v / 6.0 * e;
    fD        = fT - v * v * v * v / 30.0 * e;
  }
  G[0] = -fE * iR3;
  G[1] = 3.0 * fT * iR3 * iR2;
  G[2] = -15.0 * fD * iR3 * iR2 * iR2;
}

// Field at r (target - source) of one order-m source S; a = Thole parameter or 0.
inline void p2p(int m, double x, double y, double z, double a, const double* S, double* F) {
  double R = std::sqrt(x * x + y * y + z * z);
  double G[3];
  radial(R, a, G);
  if (m == 0) {
    double c = -S[0] * G[0];
    F[0] += c * x, F[1] += c * y, F[2] += c * z;
  } else if (m == 1) {
    double sr = S[0] * x + S[1] * y + S[2] * z;
    F[0] -= S[0] * G[0] + sr * x * G[1];
    F[1] -= S[1] * G[0] + sr * y * G[1];
    F[2] -= S[2] * G[0] + sr * z * G[1];
  } else {
    // S = (xx, xy, xz, yy, yz, zz) multi-index moments; Q = symmetric matrix
    // with the off-diagonal moments halved so that sum_k S_k X_k = Q:X.
    double qxx = S[0], qxy = 0.5 * S[1], qxz = 0.5 * S[2], qyy = S[3], qyz = 0.5 * S[4],
           qzz = S[5];
    double tr  = qxx + qyy + qzz;
    double qrx = qxx * x + qxy * y + qxz * z;
    double qry = qxy * x + qyy * y + qyz * z;
    double qrz = qxz * x + qyz * y + qzz * z;
    double rqr = x * qrx + y * qry + z * qrz;
    F[0] -= G[1] * (tr * x + 2.0 * qrx) + G[2] * rqr * x;
    F[1] -= G[1] * (tr * y + 2.0 * qry) + G[2] * rqr * y;
    F[2] -= G[1] * (tr * z + 2.0 * qrz) + G[2] * rqr * z;
  }
}

inline int ncomp(int m) { return (m + 1) * (m + 2) / 2; }

struct Site {
  double r[3];
  const int* ex;
  int nex;
  double alpha;  // isotropic polarizability used for damping, 0 if none
  bool excludes(int j) const {
    for (int e = 0; e < nex; ++e)
      if (ex[e] == j) return true;
    return false;
  }
};

struct Cell {
  double x, y, z, r, rmax;
  int parent, level;
  int child[8];
  unsigned nchild;
  int nleaf;
  std::vector<int> leaf;
};

struct Tree {
  std::vector<Cell> cells;
  std::vector<std::pair<int, int>> m2l;  // (source B, target A), sorted by source
  std::vector<std::pair<int, int>> p2p;  // (target A, source B)
};

void add_child(std::vector<Cell>& cells, int octant, int p, int ncrit) {
  const double r = cells[p].r / 2.0;
  Cell c;
  c.x      = cells[p].x + r * ((octant & 1) * 2 - 1);
  c.y      = cells[p].y + r * ((octant & 2) - 1);
  c.z      = cells[p].z + r * ((octant & 4) / 2 - 1);
  c.r      = r;
  c.rmax   = std::sqrt(3 * r * r);
  c.parent = p;
  c.level  = cells[p].level + 1;
  for (int& ch : c.child) ch = 0;
  c.nchild = 0;
  c.nleaf  = 0;
  c.leaf.assign(ncrit, 0);
  int idx = (int)cells.size();
  cells.push_back(std::move(c));
  cells[p].child[octant] = idx;
  cells[p].nchild |= (1u << octant);
}

inline int octant_of(const double* r, const Cell& c) {
  return (r[0] > c.x) + ((r[1] > c.y) << 1) + ((r[2] > c.z) << 2);
}

bool split_cell(std::vector<Cell>& cells, const std::vector<Site>& s, int p, int ncrit,
                int depth) {
  if (depth > 200) return false;  // coincident sites: the reference recurses forever
  for (int i = 0; i < ncrit; ++i) {
    int l   = cells[p].leaf[i];
    int oct = octant_of(s[l].r, cells[p]);
    if (!(cells[p].nchild & (1u << oct))) add_child(cells, oct, p, ncrit);
    int c                         = cells[p].child[oct];
    cells[c].leaf[cells[c].nleaf] = l;
    cells[c].nleaf += 1;
    if (cells[c].nleaf >= ncrit)
      if (!split_cell(cells, s, c, ncrit, depth + 1)) return false;
  }
  return true;
}

void walk(int A, int B, const std::vector<Cell>& c, double theta, int ncrit, Tree& t) {
  const double dx = c[A].x - c[B].x;
  const double dy = c[A].y - c[B].y;
  const double dz = c[A].z - c[B].z;
  // Evaluated without FMA contraction (this file is built with
  // -ffp-contract=off): cells offset by (4,4,4) half-widths sit exactly on the
  // theta = 0.5 boundary, and the reference's golden per-site FMM errors
  // (tests/ref_fmm_errors.csv, all theta/order columns) are reproduced only by
  // the uncontracted sum.
  const double R  = std::sqrt(dx * dx + dy * dy + dz * dz);
  if (R * theta > (c[A].rmax + c[B].rmax)) {
    t.m2l.push_back({B, A});
  } else if (c[A].nchild == 0 && c[B].nchild == 0) {
    if (c[B].nleaf >= ncrit)
      t.m2l.push_back({B, A});
    else
      t.p2p.push_back({A, B});
  } else if (c[B].nchild == 0 || (c[A].rmax >= c[B].rmax && c[A].nchild != 0)) {
    for (int o = 0; o < 8; ++o)
      if (c[A].nchild & (1u << o)) walk(c[A].child[o], B, c, theta, ncrit, t);
  } else {
    for (int o = 0; o < 8; ++o)
      if (c[B].nchild & (1u << o)) walk(A, c[B].child[o], c, theta, ncrit, t);
  }
}

bool build_tree(const std::vector<Site>& s, int ncrit, double theta, Tree& t) {
  const int n = (int)s.size();
  double xa = 0, ya = 0, za = 0;
  for (int i = 0; i < n; ++i) xa += s[i].r[0], ya += s[i].r[1], za += s[i].r[2];
  xa /= n, ya /= n, za /= n;
  double xm = 0, ym = 0, zm = 0;
  for (int i = 0; i < n; ++i) {
    double x = std::abs(s[i].r[0] - xa), y = std::abs(s[i].r[1] - ya),
           z = std::abs(s[i].r[2] - za);
    if (x > xm) xm = x;
    if (y > ym) ym = y;
    if (z > zm) zm = z;
  }
  double r = (xm > ym ? (xm > zm ? xm : zm) : (ym > zm ? ym : zm)) * 1.001;
  Cell root;
  root.x = xa, root.y = ya, root.z = za, root.r = r;
  root.rmax   = std::sqrt(3 * r * r);
  root.parent = 0;
  root.level  = 0;
  for (int& ch : root.child) ch = 0;
  root.nchild = 0;
  root.nleaf  = 0;
  root.leaf.assign(ncrit, 0);
  t.cells.clear();
  t.cells.push_back(root);
  for (int i = 0; i < n; ++i) {
    int cur = 0;
    while (t.cells[cur].nleaf >= ncrit) {
      t.cells[cur].nleaf += 1;
      int oct = octant_of(s[i].r, t.cells[cur]);
      if (!(t.cells[cur].nchild & (1u << oct))) add_child(t.cells, oct, cur, ncrit);
      cur = t.cells[cur].child[oct];
    }
    t.cells[cur].leaf[t.cells[cur].nleaf] = i;
    t.cells[cur].nleaf += 1;
    if (t.cells[cur].nleaf >= ncrit)
      if (!split_cell(t.cells, s, cur, ncrit, 0)) return false;
  }
  walk(0, 0, t.cells, theta, ncrit, t);
  std::stable_sort(t.m2l.begin(), t.m2l.end(),
                   [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
                     return a.first < b.first;
                   });
  return true;
}

inline double thole_a(double damping, double a1, double a2) {
  return damping / std::pow(a1 * a2, 1.0 / 6.0);
}

// Tree<m,3>::compute_field_fmm
bool field_fmm(int m, const std::vector<Site>& s, const double* S, int ncrit, int order,
               double theta, double damping, double* F) {
  const int n = (int)s.size();
  Tree t;
  if (!build_tree(s, ncrit, theta, t)) return false;
  const Ops& o = ops(m, order);
  const int nc = (int)t.cells.size();
  const int ns = ncomp(m);
  std::vector<double> M((size_t)nc * o.msize, 0.0), L((size_t)nc * o.lsize, 0.0);
  for (int i = 0; i < 3 * n; ++i) F[i] = 0.0;
  const int nt = nterms(order);

  // P2M: every particle of an unsplit cell, as an M2M shift of its source.
#pragma omp parallel for schedule(dynamic, 8)
  for (int c = 0; c < nc; ++c) {
    const Cell& C = t.cells[c];
    if (C.nleaf >= ncrit) continue;
    std::vector<double> mono(nt);
    double* Mc = &M[(size_t)c * o.msize];
    for (int q = 0; q < C.nleaf; ++q) {
      int l = C.leaf[q];
      monomials(C.x - s[l].r[0], C.y - s[l].r[1], C.z - s[l].r[2], order, mono.data());
      const double* Sl = &S[(size_t)ns * l];
      for (const Term& tm : o.p2m) Mc[tm.out] += mono[tm.w] * Sl[tm.in];
    }
  }
  // M2M: children before parents (reverse creation order).
  {
    std::vector<double> mono(nt);
    for (int c = nc - 1; c > 0; --c) {
      int p = t.cells[c].parent;
      monomials(t.cells[p].x - t.cells[c].x, t.cells[p].y - t.cells[c].y,
                t.cells[p].z - t.cells[c].z, order, mono.data());
      const double* Mc = &M[(size_t)c * o.msize];
      double* Mp       = &M[(size_t)p * o.msize];
      for (const Term& tm : o.m2m) Mp[tm.out] += mono[tm.w] * Mc[tm.in];
    }
  }
  // M2L, grouped by target cell.
  {
    std::vector<std::vector<int>> by_target(nc);
    for (auto& pr : t.m2l) by_target[pr.second].push_back(pr.first);
#pragma omp parallel for schedule(dynamic, 4)
    for (int A = 0; A < nc; ++A) {
      if (by_target[A].empty()) continue;
      std::vector<double> D(nt);
      double* LA = &L[(size_t)A * o.lsize];
      for (int B : by_target[A]) {
        derivs(t.cells[A].x - t.cells[B].x, t.cells[A].y - t.cells[B].y,
               t.cells[A].z - t.cells[B].z, order, D.data());
        const double* MB = &M[(size_t)B * o.msize];
        for (const Term& tm : o.m2l) LA[tm.out] += D[tm.w] * MB[tm.in];
      }
    }
  }
  // P2P, grouped by target leaf.
  {
    std::vector<std::vector<int>> by_target(nc);
    for (auto& pr : t.p2p) by_target[pr.first].push_back(pr.second);
#pragma omp parallel for schedule(dynamic, 4)
    for (int A = 0; A < nc; ++A) {
      const Cell& CA = t.cells[A];
      for (int B : by_target[A]) {
        const Cell& CB = t.cells[B];
        for (int p1 = 0; p1 < CA.nleaf; ++p1) {
          int l1 = CA.leaf[p1];
          for (int p2 = 0; p2 < CB.nleaf; ++p2) {
            int l2 = CB.leaf[p2];
            if (l2 == l1 || s[l1].excludes(l2)) continue;
            double a = 0.0;
            if (damping > 0.0 && s[l1].alpha > 0.0 && s[l2].alpha > 0.0)
              a = thole_a(damping, s[l1].alpha, s[l2].alpha);
            p2p(m, s[l1].r[0] - s[l2].r[0], s[l1].r[1] - s[l2].r[1], s[l1].r[2] - s[l2].r[2],
                a, &S[(size_t)ns * l2], &F[3 * l1]);
          }
        }
      }
    }
  }
  // L2L: parents before children (creation order).
  {
    std::vector<double> mono(nt);
    for (int p = 0; p < nc; ++p)
      for (int oc = 0; oc < 8; ++oc) {
        if (!(t.cells[p].nchild & (1u << oc))) continue;
        int c = t.cells[p].child[oc];
        monomials(t.cells[c].x - t.cells[p].x, t.cells[c].y - t.cells[p].y,
                  t.cells[c].z - t.cells[p].z, order - m, mono.data());
        const double* Lp = &L[(size_t)p * o.lsize];
        double* Lc       = &L[(size_t)c * o.lsize];
        for (const Term& tm : o.l2l) Lc[tm.out] += mono[tm.w] * Lp[tm.in];
      }
  }
  // L2P
#pragma omp parallel for schedule(dynamic, 8)
  for (int c = 0; c < nc; ++c) {
    const Cell& C = t.cells[c];
    if (C.nleaf >= ncrit) continue;
    std::vector<double> mono(nt);
    const double* Lc = &L[(size_t)c * o.lsize];
    for (int q = 0; q < C.nleaf; ++q) {
      int k = C.leaf[q];
      monomials(s[k].r[0] - C.x, s[k].r[1] - C.y, s[k].r[2] - C.z, order - m, mono.data());
      for (const Term& tm : o.l2p) F[3 * k + tm.out] -= mono[tm.w] * Lc[tm.in];
    }
  }
  return true;
}

// evaluate_direct{,_damping}
void field_direct(int m, const std::vector<Site>& s, const double* S, double damping,
                  double* F) {
  const int n  = (int)s.size();
  const int ns = ncomp(m);
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < n; ++i) {
    double f[3] = {0, 0, 0};
    for (int j = 0; j < n; ++j) {
      if (i == j || s[i].excludes(j)) continue;
      double a = 0.0;
      if (damping > 0.0 && std::abs(s[i].alpha) > 0.0 && std::abs(s[j].alpha) > 0.0)
        a = thole_a(damping, s[i].alpha, s[j].alpha);
      p2p(m, s[i].r[0] - s[j].r[0], s[i].r[1] - s[j].r[1], s[i].r[2] - s[j].r[2], a,
          &S[(size_t)ns * j], f);
    }
    F[3 * i] += f[0], F[3 * i + 1] += f[1], F[3 * i + 2] += f[2];
  }
}

std::vector<Site> make_sites(int n, const double* xyz, const int* pol, const double* aiso,
                             const int* ep, const int* ei, double damping) {
  std::vector<Site> s(n);
  for (int i = 0; i < n; ++i) {
    s[i].r[0]  = xyz[3 * i];
    s[i].r[1]  = xyz[3 * i + 1];
    s[i].r[2]  = xyz[3 * i + 2];
    s[i].ex    = ep ? ei + ep[i] : nullptr;
    s[i].nex   = ep ? ep[i + 1] - ep[i] : 0;
    s[i].alpha = (damping > 0.0 && pol && pol[i]) ? aiso[i] : 0.0;
  }
  return s;
}

bool field(int m, const std::vector<Site>& s, const double* S, int fmm, int ncrit, int order,
           double theta, double damping, double* F) {
  if (fmm) return field_fmm(m, s, S, ncrit, order, theta, damping, F);
  for (size_t i = 0; i < 3 * s.size(); ++i) F[i] = 0.0;
  field_direct(m, s, S, damping, F);
  return true;
}

struct BMat {
  int n;
  std::vector<Site> s;
  std::vector<double> a6, ainv;
  int fmm, ncrit, order;
  double theta, damping;
  bool apply(const double* in, double* out) const {
    std::vector<double> F(3 * (size_t)n);
    if (!field(1, s, in, fmm, ncrit, order, theta, damping, F.data())) return false;
    for (int i = 0; i < n; ++i) {
      const double* A = &ainv[9 * (size_t)i];
      const double* v = &in[3 * (size_t)i];
      for (int r = 0; r < 3; ++r)
        out[3 * i + r] = F[3 * i + r] + (A[3 * r] * v[0] + A[3 * r + 1] * v[1] + A[3 * r + 2] * v[2]);
    }
    return true;
  }
  void alpha(const double* in, double* out) const {
    for (int i = 0; i < n; ++i) {
      const double* a = &a6[6 * (size_t)i];
      const double* v = &in[3 * (size_t)i];
      out[3 * i]      = a[0] * v[0] + a[1] * v[1] + a[2] * v[2];
      out[3 * i + 1]  = a[1] * v[0] + a[3] * v[1] + a[4] * v[2];
      out[3 * i + 2]  = a[2] * v[0] + a[4] * v[1] + a[5] * v[2];
    }
  }
};

BMat make_bmat(int n, const double* xyz, const double* a6, const int* ep, const int* ei,
               int fmm, int ncrit, int order, double theta, double damping) {
  BMat B;
  B.n = n;
  std::vector<int> pol(n, 1);
  std::vector<double> iso(n);
  for (int i = 0; i < n; ++i) iso[i] = (a6[6 * i] + a6[6 * i + 3] + a6[6 * i + 5]) / 3.0;
  B.s = make_sites(n, xyz, pol.data(), iso.data(), ep, ei, damping);
  B.a6.assign(a6, a6 + 6 * (size_t)n);
  B.ainv.resize(9 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    const double* s = &a6[6 * (size_t)i];
    double a[9]     = {s[0], s[1], s[2], s[1], s[3], s[4], s[2], s[4], s[5]};
    double* o       = &B.ainv[9 * (size_t)i];
    double c0 = a[4] * a[8] - a[5] * a[7], c1 = a[5] * a[6] - a[3] * a[8],
           c2 = a[3] * a[7] - a[4] * a[6];
    double id = 1.0 / (a[0] * c0 + a[1] * c1 + a[2] * c2);
    o[0] = c0 * id, o[1] = (a[2] * a[7] - a[1] * a[8]) * id, o[2] = (a[1] * a[5] - a[2] * a[4]) * id;
    o[3] = c1 * id, o[4] = (a[0] * a[8] - a[2] * a[6]) * id, o[5] = (a[2] * a[3] - a[0] * a[5]) * id;
    o[6] = c2 * id, o[7] = (a[1] * a[6] - a[0] * a[7]) * id, o[8] = (a[0] * a[4] - a[1] * a[3]) * id;
  }
  B.fmm = fmm, B.ncrit = ncrit, B.order = order, B.theta = theta, B.damping = damping;
  return B;
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

}  // namespace orc

using namespace orc;

extern "C" {

int orc_field(int m, int n, const double* xyz, const double* S, const int* pol,
              const double* aiso, const int* ep, const int* ei, int fmm, int ncrit, int order,
              double theta, double damping, double* F) {
  if (m < 0 || m > 2) return 2;
  auto s = make_sites(n, xyz, pol, aiso, ep, ei, damping);
  return field(m, s, S, fmm, ncrit, order, theta, damping, F) ? 0 : 2;
}

int orc_multipole_fields(int n, const double* xyz, const double* q, const double* mu,
                         const double* quad, int max_order, const int* pol,
                         const double* aiso, const int* ep, const int* ei, int fmm, int ncrit,
                         int order, double theta, double damping, double* F) {
  if (max_order > 2) return 2;
  auto s = make_sites(n, xyz, pol, aiso, ep, ei, damping);
  std::vector<double> f(3 * (size_t)n);
  if (!field(0, s, q, fmm, ncrit, order, theta, damping, f.data())) return 2;
  for (size_t i = 0; i < 3 * (size_t)n; ++i) F[i] = f[i];
  if (max_order > 0) {
    if (!field(1, s, mu, fmm, ncrit, order, theta, damping, f.data())) return 2;
    for (size_t i = 0; i < 3 * (size_t)n; ++i) F[i] -= f[i];
  }
  if (max_order > 1) {
    std::vector<double> qd(quad, quad + 6 * (size_t)n);
    for (int i = 0; i < n; ++i) qd[6 * i] *= 0.5, qd[6 * i + 3] *= 0.5, qd[6 * i + 5] *= 0.5;
    if (!field(2, s, qd.data(), fmm, ncrit, order, theta, damping, f.data())) return 2;
    for (size_t i = 0; i < 3 * (size_t)n; ++i) F[i] += f[i];
  }
  return 0;
}

int orc_bmatrix_apply(int n, const double* xyz, const double* a6, const int* ep, const int* ei,
                      int fmm, int ncrit, int order, double theta, double damping,
                      const double* in, double* out) {
  BMat B = make_bmat(n, xyz, a6, ep, ei, fmm, ncrit, order, theta, damping);
  return B.apply(in, out) ? 0 : 2;
}

int orc_solve(int n, const double* xyz, const double* a6, const int* ep, const int* ei, int fmm,
              int ncrit, int order, double theta, double damping, const double* rhs_in,
              const double* guess, int make_guess, double thresh, int maxiter, double* mu,
              int* iters, double* hist) {
  BMat B          = make_bmat(n, xyz, a6, ep, ei, fmm, ncrit, order, theta, damping);
  const size_t N  = 3 * (size_t)n;
  std::vector<double> rhs(rhs_in, rhs_in + N), x(N), r(N), z(N), p(N), Ap(N), z1(N);
  if (make_guess)
    B.alpha(rhs.data(), x.data());
  else
    for (size_t i = 0; i < N; ++i) x[i] = guess ? guess[i] : 0.0;
  if (!B.apply(x.data(), Ap.data())) return 2;
  for (size_t i = 0; i < N; ++i) r[i] = rhs[i] - Ap[i];
  B.alpha(r.data(), z.data());
  p              = z;
  bool converged = false;
  int k          = 0;
  for (; k < maxiter; ++k) {
    if (!B.apply(p.data(), Ap.data())) return 2;
    double rz = dot(r, z);
    double al = rz / dot(p, Ap);
    for (size_t i = 0; i < N; ++i) x[i] += al * p[i];
    for (size_t i = 0; i < N; ++i) r[i] -= al * Ap[i];
    double rn = std::sqrt(dot(r, r));
    if (hist) hist[k] = rn;
    if (rn < thresh) {
      converged = true;
      break;
    }
    B.alpha(r.data(), z1.data());
    double be = dot(z1, r) / rz;
    for (size_t i = 0; i < N; ++i) p[i] = z1[i] + be * p[i];
    z.swap(z1);
  }
  for (size_t i = 0; i < N; ++i) mu[i] = x[i];
  if (iters) *iters = converged ? k + 1 : k;
  return converged ? 0 : 1;
}

int orc_tree_info(int n, const double* xyz, int ncrit, int order, double theta, int* ncells,
                  long* nm2l, long* np2p) {
  (void)order;
  auto s = make_sites(n, xyz, nullptr, nullptr, nullptr, nullptr, 0.0);
  Tree t;
  if (!build_tree(s, ncrit, theta, t)) return 2;
  *ncells = (int)t.cells.size();
  *nm2l   = (long)t.m2l.size();
  *np2p   = (long)t.p2p.size();
  return 0;
}

int orc_tree_lists(int n, const double* xyz, int ncrit, int order, double theta, double* cxyzr,
                   int* parent, int* level, int* nchild, int* nleaf, int* leaves, int* m2l,
                   int* p2p_out) {
  (void)order;
  auto s = make_sites(n, xyz, nullptr, nullptr, nullptr, nullptr, 0.0);
  Tree t;
  if (!build_tree(s, ncrit, theta, t)) return 2;
  for (size_t c = 0; c < t.cells.size(); ++c) {
    const Cell& C = t.cells[c];
    cxyzr[4 * c] = C.x, cxyzr[4 * c + 1] = C.y, cxyzr[4 * c + 2] = C.z, cxyzr[4 * c + 3] = C.r;
    parent[c] = C.parent, level[c] = C.level, nchild[c] = (int)C.nchild, nleaf[c] = C.nleaf;
    for (int q = 0; q < ncrit; ++q)
      leaves[c * ncrit + q] = (q < C.nleaf && C.nleaf < ncrit) ? C.leaf[q] : -1;
  }
  for (size_t i = 0; i < t.m2l.size(); ++i) m2l[2 * i] = t.m2l[i].first, m2l[2 * i + 1] = t.m2l[i].second;
  for (size_t i = 0; i < t.p2p.size(); ++i)
    p2p_out[2 * i] = t.p2p[i].first, p2p_out[2 * i + 1] = t.p2p[i].second;
  return 0;
}

}  // extern "C"
