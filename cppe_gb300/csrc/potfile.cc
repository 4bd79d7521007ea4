// Potfile ingest straight into the arrays the C ABI takes: positions,
// multipoles up to order 2, polarizabilities and the exclusion lists as CSR
// (cppe_gpu_create's excl_ptr / excl_idx).  Same file format, unit
// conversion, trace removal, defaults and error messages as the reference's
// PotfileReader::read (src/core/potfile_reader.cc:31-179), without the
// per-site objects: the file is read into memory once, scanned line by line
// with locale-free number parsing, and the exclusion lists are counted and
// then scattered into one CSR array (no per-site vectors, no per-pair lookups).
#include <algorithm>
#include <cctype>
#include <charconv>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "cppe_gpu.h"

namespace cg {
void set_last_error(const std::string& msg);
}

struct cppe_gpu_potfile {
  int n         = 0;
  int max_order = -1;  // highest multipole order present (-1: none)
  std::vector<double> xyz, q, mu, quad, alpha6;
  std::vector<int> polarizable, excl_ptr, excl_idx;
  std::vector<char> elements;  // n x 4, NUL-padded element symbols
};

namespace {

const double kAngToBohr = 1.8897261246;  // potfile_reader.cc:22

struct Lines {
  std::string buf;
  size_t pos = 0;
  bool next(std::string_view& line) {
    if (pos >= buf.size()) return false;
    size_t e = buf.find('\n', pos);
    if (e == std::string::npos) e = buf.size();
    line = std::string_view(buf).substr(pos, e - pos);
    if (!line.empty() && line.back() == '\r') line.remove_suffix(1);
    pos = e + 1;
    return true;
  }
  std::string_view must(void) {
    std::string_view l;
    if (!next(l)) throw std::runtime_error("unexpected end of potential file");
    return l;
  }
};

// splits a line into at most `cap` whitespace-separated tokens; returns the count
int split(std::string_view line, std::string_view* t, int cap) {
  int k = 0;
  size_t i = 0;
  const size_t n = line.size();
  while (i < n) {
    while (i < n && std::isspace((unsigned char)line[i])) ++i;
    size_t j = i;
    while (j < n && !std::isspace((unsigned char)line[j])) ++j;
    if (j > i) {
      if (k == cap) return cap + 1;
      t[k++] = line.substr(i, j - i);
    }
    i = j;
  }
  return k;
}

double num(std::string_view t) {
  if (!t.empty() && t[0] == '+') t.remove_prefix(1);
  double v = 0.0;
  const auto rc = std::from_chars(t.data(), t.data() + t.size(), v);
  if (rc.ec != std::errc() || rc.ptr != t.data() + t.size())
    throw std::invalid_argument("invalid number in potential file: " + std::string(t));
  return v;
}

long inum(std::string_view t) {
  if (!t.empty() && t[0] == '+') t.remove_prefix(1);
  long v = 0;
  const auto rc = std::from_chars(t.data(), t.data() + t.size(), v);
  if (rc.ec != std::errc()) throw std::invalid_argument("invalid integer in potential file");
  return v;
}

int site_index(std::string_view t, int n) {
  const long s = inum(t) - 1;
  if (s < 0 || s >= n) throw std::out_of_range("site index out of range in potential file");
  return (int)s;
}

void read_file(const char* path, cppe_gpu_potfile& P) {
  Lines L;
  {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error("Potential file does not exist.");
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    L.buf.resize(size > 0 ? (size_t)size : 0);
    const size_t got = size > 0 ? std::fread(&L.buf[0], 1, (size_t)size, f) : 0;
    std::fclose(f);
    if (got != L.buf.size()) throw std::runtime_error("could not read the potential file");
  }
  std::string_view line, t[16];
  std::vector<int> ex_site, ex_val;  // exclusion pairs in file order
  bool have_coords = false;
  while (L.next(line)) {
    if (line.find("@COORDINATES") != std::string_view::npos) {
      if (split(L.must(), t, 16) < 1) throw std::runtime_error("missing site count");
      const long n = inum(t[0]);
      if (n < 0 || n > (1L << 30)) throw std::invalid_argument("invalid site count");
      const int nu = split(L.must(), t, 16);
      const std::string unit = nu >= 1 ? std::string(t[0]) : std::string();
      double conv;
      if (unit == "AA")
        conv = kAngToBohr;
      else if (unit == "AU")
        conv = 1.0;
      else
        throw std::runtime_error("Invalid unit for potential file.");
      P.n = (int)n;
      P.xyz.resize(3 * (size_t)n);
      P.elements.assign(4 * (size_t)n, 0);
      for (long i = 0; i < n; ++i) {
        if (split(L.must(), t, 16) < 4) throw std::runtime_error("malformed coordinate line");
        for (int c = 0; c < 3; ++c) P.xyz[3 * i + c] = num(t[1 + c]) * conv;
        std::memcpy(&P.elements[4 * i], t[0].data(), std::min<size_t>(3, t[0].size()));
      }
      P.q.assign(n, 0.0), P.mu.assign(3 * (size_t)n, 0.0), P.quad.assign(6 * (size_t)n, 0.0);
      P.alpha6.assign(6 * (size_t)n, 0.0), P.polarizable.assign(n, 0);
      have_coords = true;
    }
    if (line.find("ORDER") != std::string_view::npos) {
      std::string_view h[4];
      const int nh = split(line, h, 3);
      if (!have_coords) throw std::runtime_error("ORDER section before @COORDINATES");
      if (nh == 2) {
        const long order = inum(h[1]);
        if (order < 0 || order > 2)
          throw std::invalid_argument("multipoles above order 2 are not supported");
        const int ncomp = (int)((order + 1) * (order + 2) / 2);
        split(L.must(), t, 16);
        const long count = inum(t[0]);
        P.max_order      = std::max<int>(P.max_order, (int)order);
        double* dst = order == 0 ? P.q.data() : order == 1 ? P.mu.data() : P.quad.data();
        for (long k = 0; k < count; ++k) {
          if (split(L.must(), t, 16) < 1 + ncomp) throw std::runtime_error("malformed multipole line");
          const int s = site_index(t[0], P.n);
          double v[6];
          for (int c = 0; c < ncomp; ++c) v[c] = num(t[1 + c]);
          if (order == 2) {  // Multipole::remove_trace (potential.hh)
            const double tr = (v[0] + v[3] + v[5]) / 3.0;
            v[0] -= tr, v[3] -= tr, v[5] -= tr;
          }
          for (int c = 0; c < ncomp; ++c) dst[(size_t)s * ncomp + c] = v[c];
        }
      } else if (nh == 3) {
        if (inum(h[1]) != 1 || inum(h[2]) != 1)
          throw std::runtime_error("Only dipole-dipole polarizabilities are currently supported.");
        split(L.must(), t, 16);
        const long count = inum(t[0]);
        for (long k = 0; k < count; ++k) {
          if (split(L.must(), t, 16) < 7) throw std::runtime_error("malformed polarizability line");
          const int s = site_index(t[0], P.n);
          if (P.polarizable[s])
            throw std::runtime_error("Potential can only have one polarizability.");
          for (int c = 0; c < 6; ++c) P.alpha6[6 * (size_t)s + c] = num(t[1 + c]);
          P.polarizable[s] = 1;
        }
      } else {
        throw std::runtime_error("Invalid number in potfile ORDER.");
      }
    }
    if (line.find("EXCLISTS") != std::string_view::npos) {
      if (!have_coords) throw std::runtime_error("EXCLISTS before @COORDINATES");
      split(L.must(), t, 16);
      const long count = inum(t[0]);
      for (long k = 0; k < count; ++k) {
        std::string_view el = L.must();
        // split without a token cap (exclusion lists may be long)
        size_t i = 0;
        int s = -1;
        while (i < el.size()) {
          while (i < el.size() && std::isspace((unsigned char)el[i])) ++i;
          size_t j = i;
          while (j < el.size() && !std::isspace((unsigned char)el[j])) ++j;
          if (j > i) {
            const std::string_view tok = el.substr(i, j - i);
            if (s < 0) {
              s = site_index(tok, P.n);
            } else {
              const long e = inum(tok) - 1;  // 0 entries pad the lists
              if (e >= 0) ex_site.push_back(s), ex_val.push_back((int)e);
            }
          }
          i = j;
        }
      }
    }
  }
  // exclusions: count per site, prefix sum, scatter in file order
  P.excl_ptr.assign((size_t)P.n + 1, 0);
  for (int s : ex_site) ++P.excl_ptr[s + 1];
  for (int i = 0; i < P.n; ++i) P.excl_ptr[i + 1] += P.excl_ptr[i];
  P.excl_idx.resize(ex_val.size());
  std::vector<int> fill(P.excl_ptr.begin(), P.excl_ptr.end() - 1);
  for (size_t k = 0; k < ex_val.size(); ++k) P.excl_idx[fill[ex_site[k]]++] = ex_val[k];
}

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const std::invalid_argument& e) {
    cg::set_last_error(e.what());
    return CPPE_GPU_INVALID_ARG;
  } catch (const std::out_of_range& e) {
    cg::set_last_error(e.what());
    return CPPE_GPU_INVALID_ARG;
  } catch (const std::exception& e) {
    cg::set_last_error(e.what());
    return CPPE_GPU_INVALID_ARG;
  }
}

template <class T>
void copy_out(const std::vector<T>& v, T* dst) {
  if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
}

}  // namespace

extern "C" {

int cppe_gpu_potfile_read(const char* path, cppe_gpu_potfile** out) {
  return guarded([&]() -> int {
    if (!path || !out) throw std::invalid_argument("null argument");
    *out  = nullptr;
    auto* P = new cppe_gpu_potfile();
    try {
      read_file(path, *P);
    } catch (...) {
      delete P;
      throw;
    }
    *out = P;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_potfile_info(const cppe_gpu_potfile* p, int* n, int* max_order, int* npolarizable,
                          long* nexcl) {
  return guarded([&]() -> int {
    if (!p) throw std::invalid_argument("null potfile");
    if (n) *n = p->n;
    if (max_order) *max_order = p->max_order;
    if (npolarizable)
      *npolarizable = (int)std::count(p->polarizable.begin(), p->polarizable.end(), 1);
    if (nexcl) *nexcl = (long)p->excl_idx.size();
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_potfile_arrays(const cppe_gpu_potfile* p, double* xyz, double* q, double* mu,
                            double* quad, double* alpha6, int* polarizable, int* excl_ptr,
                            int* excl_idx, char* elements) {
  return guarded([&]() -> int {
    if (!p) throw std::invalid_argument("null potfile");
    copy_out(p->xyz, xyz), copy_out(p->q, q), copy_out(p->mu, mu), copy_out(p->quad, quad);
    copy_out(p->alpha6, alpha6), copy_out(p->polarizable, polarizable);
    copy_out(p->excl_ptr, excl_ptr), copy_out(p->excl_idx, excl_idx);
    copy_out(p->elements, elements);
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_potfile_free(cppe_gpu_potfile* p) {
  delete p;
  return CPPE_GPU_OK;
}

}  // extern "C"
