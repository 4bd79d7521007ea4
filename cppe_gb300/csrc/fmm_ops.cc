// Construction of the Cartesian FMM operator index tables (see fmm_ops.h).
#include "fmm_ops.h"

#include <algorithm>
#include <array>
#include <stdexcept>

namespace cg {

namespace {
struct MultiIndex {
  std::vector<int> a, b, c;
  int at[PMAX + 2][PMAX + 2][PMAX + 2];
  MultiIndex() {
    for (int o = 0; o <= PMAX + 1; ++o)
      for (int x = o; x >= 0; --x)
        for (int y = o - x; y >= 0; --y) {
          at[x][y][o - x - y] = (int)a.size();
          a.push_back(x), b.push_back(y), c.push_back(o - x - y);
        }
  }
  int idx(int x, int y, int z) const { return at[x][y][z]; }
};
const MultiIndex& MI() {
  static const MultiIndex mi;
  return mi;
}
}  // namespace

OpTables make_op_tables(int m, int p) {
  if (m < 0 || m > 2 || p < m || p > PMAX) throw std::invalid_argument("bad FMM order");
  const MultiIndex& I = MI();
  OpTables o;
  o.m     = m;
  o.p     = p;
  o.moff  = nterms(m - 1);
  o.nt    = nterms(p);
  o.msize = o.nt - o.moff;
  o.lsize = nterms(p - m);
  for (int j = 0; j < o.nt; ++j) o.exps.push_back(I.a[j] | (I.b[j] << 4) | (I.c[j] << 8));

  auto sub = [&](int n, int k, int& j) {
    int x = I.a[n] - I.a[k], y = I.b[n] - I.b[k], z = I.c[n] - I.c[k];
    if (x < 0 || y < 0 || z < 0) return false;
    j = I.idx(x, y, z);
    return true;
  };
  // P2M and M2M rows
  o.p2m_ptr.push_back(0);
  o.m2m_ptr.push_back(0);
  for (int n = o.moff; n < o.nt; ++n) {
    for (int k = o.moff; k <= n; ++k) {
      int j;
      if (!sub(n, k, j)) continue;
      o.m2m_k.push_back(k - o.moff), o.m2m_j.push_back(j);
      if (k < nterms(m)) o.p2m_k.push_back(k - o.moff), o.p2m_j.push_back(j);
    }
    o.p2m_ptr.push_back((int)o.p2m_k.size());
    o.m2m_ptr.push_back((int)o.m2m_k.size());
  }
  // L2L rows
  o.l2l_ptr.push_back(0);
  for (int n = 0; n < o.lsize; ++n) {
    for (int k = n; k < o.lsize; ++k) {
      int j;
      if (sub(k, n, j)) o.l2l_k.push_back(k), o.l2l_j.push_back(j);
    }
    o.l2l_ptr.push_back((int)o.l2l_k.size());
  }
  // L2P
  for (int c = 0; c < 3; ++c)
    for (int n = 1; n < o.lsize; ++n) {
      int e[3] = {I.a[n], I.b[n], I.c[n]};
      if (e[c] == 0) continue;
      e[c] -= 1;
      o.l2p_c.push_back(c), o.l2p_n.push_back(n), o.l2p_j.push_back(I.idx(e[0], e[1], e[2]));
    }
  // M2L terms
  std::vector<int> row_begin;
  for (int n = 0; n < o.lsize; ++n) {
    row_begin.push_back((int)o.m2l_row.size());
    int on = I.a[n] + I.b[n] + I.c[n];
    for (int k = o.moff; k < nterms(p - on); ++k) {
      o.m2l_row.push_back(n);
      o.m2l_k.push_back(k - o.moff);
      o.m2l_w.push_back(I.idx(I.a[n] + I.a[k], I.b[n] + I.b[k], I.c[n] + I.c[k]));
    }
  }
  row_begin.push_back((int)o.m2l_row.size());
  // Slot schedule: cut rows into segments no longer than `cap`, then give each
  // segment to the least-loaded lane that still has a free slot.
  const int total = (int)o.m2l_row.size();
  int cap         = std::max(1, (total + 31) / 32);
  for (;; ++cap) {
    std::vector<std::array<int, 3>> segs;
    for (int n = 0; n < o.lsize; ++n)
      for (int t0 = row_begin[n]; t0 < row_begin[n + 1]; t0 += cap)
        segs.push_back({n, t0, std::min(t0 + cap, row_begin[n + 1])});
    std::vector<int> load(32, 0), used(32, 0);
    std::vector<int> slots(32 * M2L_SLOTS * 3, 0);
    for (int l = 0; l < 32; ++l)
      for (int s = 0; s < M2L_SLOTS; ++s) {
        slots[(l * M2L_SLOTS + s) * 3 + 0] = 0;
        slots[(l * M2L_SLOTS + s) * 3 + 1] = 0;
        slots[(l * M2L_SLOTS + s) * 3 + 2] = 0;  // empty slot: t0 == t1
      }
    // longest first
    std::vector<int> order(segs.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      return segs[a][2] - segs[a][1] > segs[b][2] - segs[b][1];
    });
    bool ok = true;
    std::vector<std::vector<int>> row_slots(o.lsize);
    for (int si : order) {
      int best = -1;
      for (int l = 0; l < 32; ++l)
        if (used[l] < M2L_SLOTS && (best < 0 || load[l] < load[best])) best = l;
      if (best < 0) {
        ok = false;
        break;
      }
      int id            = best * M2L_SLOTS + used[best]++;
      slots[id * 3 + 0] = segs[si][0];
      slots[id * 3 + 1] = segs[si][1];
      slots[id * 3 + 2] = segs[si][2];
      load[best] += segs[si][2] - segs[si][1];
      row_slots[segs[si][0]].push_back(id);
    }
    if (!ok) continue;
    o.slots = slots;
    o.row_slot_ptr.assign(1, 0);
    o.row_slot_id.clear();
    for (int n = 0; n < o.lsize; ++n) {
      std::sort(row_slots[n].begin(), row_slots[n].end(), [&](int a, int b) {
        return slots[a * 3 + 1] < slots[b * 3 + 1];
      });
      for (int id : row_slots[n]) o.row_slot_id.push_back(id);
      o.row_slot_ptr.push_back((int)o.row_slot_id.size());
    }
    break;
  }
  // Derivative recurrence
  o.drec.assign(8 * (size_t)o.nt, -1);
  for (int j = 1; j < o.nt; ++j) {
    int n[3] = {I.a[j], I.b[j], I.c[j]};
    for (int i = 0; i < 3; ++i) {
      if (n[i] >= 1) {
        int q[3] = {n[0], n[1], n[2]};
        q[i] -= 1;
        o.drec[8 * j + i] = I.idx(q[0], q[1], q[2]);
      }
      if (n[i] >= 2) {
        int q[3] = {n[0], n[1], n[2]};
        q[i] -= 2;
        o.drec[8 * j + 3 + i] = I.idx(q[0], q[1], q[2]);
      }
    }
    o.drec[8 * j + 6] = n[0] + n[1] + n[2];
  }
  return o;
}

}  // namespace cg
