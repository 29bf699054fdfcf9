// sbdgb/tpb.hpp -- header-only C++ mirror of the reference's TPB entry points
// over the engine's C ABI (sbdgb.h).  A program that calls
//   sbd::tpb::generate_sbd_data / sbd::tpb::diag / sbd::LoadFCIDump /
//   sbd::LoadAlphaDets / sbd::makeQChamDiagTerms / sbd::mult / sbd::Davidson
// switches to the GB300 engine by calling the same names in namespace sbdgb.
//
// Reference interfaces mirrored (paths inside the reference project):
//   SBD options + argv parsing ....... chemistry/tpb/sbdiag.h:24-134
//   diag ............................. chemistry/tpb/sbdiag.h:151-526
//   FCIDump / LoadFCIDump ............ framework/fcidump.h:20-95
//   SetupIntegrals ................... chemistry/basic/makeintegrals.h:123-174
//   LoadAlphaDets / sort_bitarray .... chemistry/basic/makedeterminants.h:167-191,
//                                      framework/bit_manipulation.h:386-439
//   makeQChamDiagTerms ............... chemistry/tpb/qcham.h:289-340
//   mult (Wb += H Wk) ................ chemistry/tpb/mult.h:114-130
//   Davidson ......................... chemistry/tpb/davidson.h:707-726
//   MultBase::run (device operator) .. chemistry/basic/mult.h:19-103
//
// Errors: the C status codes become std::invalid_argument (bad input) or
// std::runtime_error (everything else), the exception types the reference
// throws (helper.h:361-364, davidson.h:97-110).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "sbdgb.h"

namespace sbdgb {

inline void check(int rc, const sbdgb_ctx *ctx, const char *what) {
  if (rc == SBDGB_OK) return;
  std::string msg = std::string(what) + ": " + (ctx ? sbdgb_last_error(ctx) : "error");
  if (rc == SBDGB_E_INPUT) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

// ---- FCIDUMP (framework/fcidump.h) ---------------------------------------------

struct FCIDump {
  std::map<std::string, std::string> header;
  std::vector<std::tuple<double, int, int, int, int>> integrals;
};

inline FCIDump LoadFCIDump(const std::string &filename) {
  FCIDump d;
  std::ifstream in(filename);
  if (!in.is_open()) throw std::runtime_error("Failed to open FCIDUMP file.");
  std::string line, head;
  bool in_header = true;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '!') continue;
    if (in_header) {
      if (line.find("&END") != std::string::npos) {
        in_header = false;
        continue;
      }
      size_t pos = line.find("&FCI");
      if (pos != std::string::npos) line.erase(pos, 4);
      head += line;
    } else {
      std::stringstream ss(line);
      double v;
      int i, j, k, l;
      ss >> v >> i >> j >> k >> l;
      d.integrals.emplace_back(v, i, j, k, l);
    }
  }
  std::stringstream hs(head);
  std::string tok;
  while (std::getline(hs, tok, ',')) {
    size_t eq = tok.find('=');
    if (eq == std::string::npos) continue;
    std::string key = tok.substr(0, eq), val = tok.substr(eq + 1);
    auto trim = [](std::string &s) {
      s.erase(0, s.find_first_not_of(" \t"));
      s.erase(s.find_last_not_of(" \t") + 1);
    };
    trim(key);
    trim(val);
    d.header[key] = val;
  }
  return d;
}

// Spatial integrals in the engine's layout: h1 (L*L) and the 8-fold packed ERI.
struct Integrals {
  int L = 0, N = 0;
  double I0 = 0.0;
  std::vector<double> h1, eri;
};

inline size_t pair_index(int i, int j) {
  int a = std::max(i, j), b = std::min(i, j);
  return (size_t)a * (a + 1) / 2 + b;
}

// SetupIntegrals (makeintegrals.h:123-174): core, one-body (symmetrised), two-body
// (8-fold packed); later lines overwrite earlier ones.
inline Integrals SetupIntegrals(const FCIDump &d) {
  Integrals t;
  for (const auto &kv : d.header) {
    if (kv.first == "NORB") t.L = std::atoi(kv.second.c_str());
    if (kv.first == "NELEC") t.N = std::atoi(kv.second.c_str());
  }
  if (t.L <= 0) throw std::invalid_argument("FCIDUMP header has no NORB");
  const size_t B = (size_t)t.L * (t.L + 1) / 2;
  t.h1.assign((size_t)t.L * t.L, 0.0);
  t.eri.assign(B * (B + 1) / 2, 0.0);
  for (const auto &e : d.integrals) {
    const double v = std::get<0>(e);
    const int i = std::get<1>(e), j = std::get<2>(e), k = std::get<3>(e), l = std::get<4>(e);
    if (i == 0 && j == 0 && k == 0 && l == 0) {
      t.I0 = v;
    } else if (k == 0 && l == 0) {
      if (i < 1 || j < 1 || i > t.L || j > t.L) throw std::invalid_argument("FCIDUMP one-body index out of range");
      t.h1[(size_t)(i - 1) * t.L + (j - 1)] = v;
      t.h1[(size_t)(j - 1) * t.L + (i - 1)] = v;
    } else {
      if (i < 1 || j < 1 || k < 1 || l < 1 || i > t.L || j > t.L || k > t.L || l > t.L)
        throw std::invalid_argument("FCIDUMP two-body index out of range");
      size_t ij = pair_index(i - 1, j - 1), kl = pair_index(k - 1, l - 1);
      size_t a = std::max(ij, kl), b = std::min(ij, kl);
      t.eri[a * (a + 1) / 2 + b] = v;
    }
  }
  return t;
}

// ---- strings (framework/bit_manipulation.h) -------------------------------------

// Text line -> uint64, character s[L-1-i] is orbital i (bit_manipulation.h:219-233).
inline uint64_t from_string(const std::string &s, int L) {
  if ((int)s.size() < L) throw std::invalid_argument("bit string shorter than norb");
  uint64_t v = 0;
  for (int i = 0; i < L; ++i)
    if (s[L - 1 - i] == '1') v |= 1ull << i;
  return v;
}

// Sorted, duplicate-free list: the reference's from-back order is numeric order.
inline std::vector<uint64_t> LoadAlphaDets(const std::string &file, int L) {
  if (L > 64) throw std::invalid_argument("norb > 64 is not supported");
  std::ifstream in(file);
  if (!in.is_open()) throw std::runtime_error("Failed to open alpha det file.");
  std::vector<uint64_t> v;
  std::string line;
  while (std::getline(in, line)) v.push_back(from_string(line, L));
  std::sort(v.begin(), v.end());
  v.erase(std::unique(v.begin(), v.end()), v.end());
  return v;
}

// Converts any reference-style string container (rows of `bit_length`-bit
// words, e.g. sbd::det_vector<size_t, det_kind::half>) to uint64 strings.
template <class DetVec>
std::vector<uint64_t> pack_strings(const DetVec &dets, size_t bit_length, int L) {
  std::vector<uint64_t> v(dets.size(), 0);
  const size_t words = (L + bit_length - 1) / bit_length;
  for (size_t i = 0; i < dets.size(); ++i)
    for (size_t w = 0; w < words; ++w) v[i] |= (uint64_t)dets[i][w] << (w * bit_length);
  return v;
}

// The reverse: uint64 strings to rows of `bit_length`-bit words (row-major,
// ceil(L / bit_length) words per string).
inline std::vector<size_t> to_words(const std::vector<uint64_t> &v, int L, size_t bit_length) {
  const size_t words = ((size_t)L + bit_length - 1) / bit_length;
  const uint64_t mask = bit_length >= 64 ? ~0ull : ((1ull << bit_length) - 1ull);
  std::vector<size_t> out(v.size() * words, 0);
  for (size_t i = 0; i < v.size(); ++i)
    for (size_t w = 0; w < words; ++w) out[i * words + w] = (size_t)((v[i] >> (w * bit_length)) & mask);
  return out;
}

// ---- engine objects ------------------------------------------------------------

class Context {
 public:
  explicit Context(int device = 0, size_t hbm_budget = 0) {
    check(sbdgb_ctx_create(&ctx_, device, hbm_budget), nullptr, "sbdgb_ctx_create");
  }
  ~Context() { sbdgb_ctx_destroy(ctx_); }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  sbdgb_ctx *get() const { return ctx_; }

 private:
  sbdgb_ctx *ctx_ = nullptr;
};

class Problem {
 public:
  Problem(Context &ctx, const Integrals &ints, const std::vector<uint64_t> &adet, const std::vector<uint64_t> &bdet)
      : ctx_(ctx) {
    check(sbdgb_problem_create(ctx.get(), ints.L, adet.data(), adet.size(), bdet.data(), bdet.size(),
                               ints.h1.data(), ints.eri.data(), ints.I0, &p_),
          ctx.get(), "sbdgb_problem_create");
    N_ = adet.size() * bdet.size();
  }
  ~Problem() { sbdgb_problem_destroy(p_); }
  Problem(const Problem &) = delete;
  Problem &operator=(const Problem &) = delete;
  sbdgb_problem *get() const { return p_; }
  size_t size() const { return N_; }
  sbdgb_ctx *ctx() const { return ctx_.get(); }

 private:
  Context &ctx_;
  sbdgb_problem *p_ = nullptr;
  size_t N_ = 0;
};

// makeQChamDiagTerms (qcham.h:289-340).
inline void makeQChamDiagTerms(Problem &p, std::vector<double> &hii) {
  hii.resize(p.size());
  check(sbdgb_diag_terms(p.get(), hii.data()), p.ctx(), "makeQChamDiagTerms");
}

// mult (mult.h:114-130): Wb += H * Wk on host vectors.
inline void mult(const std::vector<double> &hii, const std::vector<double> &Wk, std::vector<double> &Wb,
                 Problem &p) {
  if (Wk.size() != p.size() || Wb.size() != p.size()) throw std::invalid_argument("vector size mismatch");
  check(sbdgb_mult_host(p.get(), hii.empty() ? nullptr : hii.data(), Wk.data(), Wb.data()), p.ctx(), "mult");
}

// Davidson (davidson.h:707-726): W in = starting vector (or empty for the
// reference's init 0 guess), out = normalized ground-state vector.
inline double Davidson(Problem &p, std::vector<double> &W, int max_iteration, int num_block, double eps,
                       double max_time = 86400.0, int init = -1) {
  sbdgb_davidson_opts o;
  sbdgb_davidson_default_opts(&o);
  o.max_it = max_iteration;
  o.max_nb = num_block;
  o.eps = eps;
  o.max_time = max_time;
  o.nroots = 1;
  if (init >= 0) {
    o.init = init;
  } else {
    o.init = W.size() == p.size() ? 2 : 0;
  }
  W.resize(p.size());
  double E = 0.0;
  sbdgb_report rep;
  check(sbdgb_davidson(p.get(), &o, &E, W.data(), &rep), p.ctx(), "Davidson");
  return E;
}

// SaveWavefunction (restart.h:21-67) at communicator size 1: file + "000000"
// holding na, nb, det_length, the strings in bit_length-bit words, and W.
inline void SaveWavefunction(const std::string &file, const std::vector<uint64_t> &adet,
                             const std::vector<uint64_t> &bdet, int L, const std::vector<double> &W,
                             size_t bit_length = 20) {
  if (W.size() != adet.size() * bdet.size()) throw std::invalid_argument("SaveWavefunction: size mismatch");
  std::ofstream f(file + "000000", std::ios::binary);
  if (!f) throw std::runtime_error("SaveWavefunction: cannot open " + file + "000000");
  const size_t na = adet.size(), nb = bdet.size(), dl = ((size_t)L + bit_length - 1) / bit_length;
  f.write((const char *)&na, sizeof(size_t));
  f.write((const char *)&nb, sizeof(size_t));
  f.write((const char *)&dl, sizeof(size_t));
  auto put = [&](const std::vector<uint64_t> &v) {
    std::vector<size_t> w = to_words(v, L, bit_length);
    f.write((const char *)w.data(), (std::streamsize)(sizeof(size_t) * w.size()));
  };
  put(adet);
  put(bdet);
  f.write((const char *)W.data(), (std::streamsize)(sizeof(double) * W.size()));
}

// LoadWavefunction (restart.h:415-660) at communicator size 1: the saved
// coefficients of the (alpha, beta) pairs whose strings are in adet x bdet,
// placed at those determinants, the rest zero, normalised.
inline void LoadWavefunction(const std::string &file, const std::vector<uint64_t> &adet,
                             const std::vector<uint64_t> &bdet, std::vector<double> &W, size_t bit_length = 20) {
  std::ifstream f(file + "000000", std::ios::binary);
  if (!f) throw std::runtime_error("LoadWavefunction: cannot open " + file + "000000");
  size_t na = 0, nb = 0, dl = 0;
  f.read((char *)&na, sizeof(size_t));
  f.read((char *)&nb, sizeof(size_t));
  f.read((char *)&dl, sizeof(size_t));
  auto get = [&](size_t n) {
    std::vector<size_t> w(n * dl);
    f.read((char *)w.data(), (std::streamsize)(sizeof(size_t) * w.size()));
    std::vector<uint64_t> v(n, 0);
    for (size_t i = 0; i < n; ++i)
      for (size_t k = 0; k < dl; ++k) v[i] |= (uint64_t)w[i * dl + k] << (k * bit_length);
    return v;
  };
  const std::vector<uint64_t> la = get(na), lb = get(nb);
  std::vector<double> lw(na * nb);
  f.read((char *)lw.data(), (std::streamsize)(sizeof(double) * lw.size()));
  if (!f) throw std::runtime_error("LoadWavefunction: truncated file");
  auto index = [](const std::vector<uint64_t> &list, uint64_t x) -> long {
    auto it = std::lower_bound(list.begin(), list.end(), x);
    return (it != list.end() && *it == x) ? (long)(it - list.begin()) : -1;
  };
  W.assign(adet.size() * bdet.size(), 0.0);
  std::vector<long> jb(nb);
  for (size_t ib = 0; ib < nb; ++ib) jb[ib] = index(bdet, lb[ib]);
  for (size_t ia = 0; ia < na; ++ia) {
    const long ja = index(adet, la[ia]);
    if (ja < 0) continue;
    for (size_t ib = 0; ib < nb; ++ib)
      if (jb[ib] >= 0) W[(size_t)ja * bdet.size() + (size_t)jb[ib]] += lw[ia * nb + ib];
  }
  double n2 = 0.0;
  for (double x : W) n2 += x * x;
  if (n2 > 0.0) {
    const double inv = 1.0 / std::sqrt(n2);
    for (double &x : W) x *= inv;
  }
}

// Lanczos (lanczos.h:169-320): W in = starting vector (or empty for the
// reference's init 0 guess), out = Ritz vector; returns the energy.
inline double Lanczos(Problem &p, std::vector<double> &W, int max_iteration, int num_block, double eps) {
  sbdgb_davidson_opts o;
  sbdgb_davidson_default_opts(&o);
  o.max_it = max_iteration;
  o.max_nb = num_block;
  o.eps = eps;
  o.nroots = 1;
  o.init = W.size() == p.size() ? 2 : 0;
  W.resize(p.size());
  double E = 0.0;
  sbdgb_report rep;
  check(sbdgb_lanczos(p.get(), &o, &E, W.data(), &rep), p.ctx(), "Lanczos");
  return E;
}

// Many small problems of one context solved in lock step (no reference
// counterpart; sbdgb_batch_davidson).  Returns energies[i][r] for problem i and
// root r; precision SBDGB_MIXED runs an FP32 phase before the FP64 phase.
inline std::vector<std::vector<double>> BatchDavidson(std::vector<Problem *> &problems, int nroots, int num_block,
                                                      double eps, int max_iteration = 100,
                                                      int precision = SBDGB_FP64) {
  std::vector<std::vector<double>> out(problems.size());
  if (problems.empty()) return out;
  sbdgb_davidson_opts o;
  sbdgb_davidson_default_opts(&o);
  o.max_it = max_iteration;
  o.max_nb = num_block;
  o.eps = eps;
  o.nroots = nroots;
  o.init = 1;
  o.precision = precision;
  std::vector<sbdgb_problem *> ps(problems.size());
  for (size_t i = 0; i < problems.size(); ++i) {
    if (problems[i]->ctx() != problems[0]->ctx()) throw std::invalid_argument("batch problems share one context");
    ps[i] = problems[i]->get();
  }
  std::vector<double> E(problems.size() * nroots);
  check(sbdgb_batch_davidson(problems[0]->ctx(), ps.data(), (int)ps.size(), &o, E.data(), nullptr, nullptr),
        problems[0]->ctx(), "BatchDavidson");
  for (size_t i = 0; i < problems.size(); ++i) out[i].assign(E.begin() + i * nroots, E.begin() + (i + 1) * nroots);
  return out;
}

// OccupationDensity (occupation.h:11-95) over all orbitals: res[2p] alpha,
// res[2p+1] beta occupation of orbital p in W.
inline void OccupationDensity(Problem &p, int norb, const std::vector<double> &W, std::vector<double> &res) {
  if (W.size() != p.size()) throw std::invalid_argument("vector size mismatch");
  res.assign(2 * (size_t)norb, 0.0);
  check(sbdgb_occupation_density(p.get(), W.data(), res.data(), nullptr), p.ctx(), "OccupationDensity");
}

// Correlation (correlation.h:379-640): one-particle (2 x L^2) and
// two-particle (4 x L^4) reduced density matrices of W in the reference layout.
inline void Correlation(Problem &p, int norb, const std::vector<double> &W, std::vector<std::vector<double>> &onebody,
                        std::vector<std::vector<double>> &twobody) {
  if (W.size() != p.size()) throw std::invalid_argument("vector size mismatch");
  const size_t L2 = (size_t)norb * norb, L4 = L2 * L2;
  std::vector<double> one(2 * L2), two(4 * L4);
  check(sbdgb_rdm(p.get(), W.data(), one.data(), two.data(), nullptr), p.ctx(), "Correlation");
  onebody.assign(2, std::vector<double>());
  twobody.assign(4, std::vector<double>());
  for (int k = 0; k < 2; ++k) onebody[k].assign(one.begin() + k * L2, one.begin() + (k + 1) * L2);
  for (int k = 0; k < 4; ++k) twobody[k].assign(two.begin() + k * L4, two.begin() + (k + 1) * L4);
}

// Carry-over selection (CarryOverAdet/Bdet, rdmat.h:62-135, 189-261): the
// strings ranked by weight sum |W|^2 (ties by index), either up to the one
// whose cumulative weight exceeds 1 - threshold or the `kept` heaviest.
inline std::vector<uint64_t> carry_over_select(const std::vector<uint64_t> &strs, const std::vector<double> &w,
                                               double threshold, size_t kept, double *discarded) {
  std::vector<size_t> order(strs.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return w[x] > w[y]; });
  size_t n = 0;
  double acc = 0.0;
  if (kept == (size_t)-1) {
    for (; n < order.size(); ++n) {
      acc += w[order[n]];
      if (acc > 1.0 - threshold) {
        ++n;
        break;
      }
    }
  } else {
    n = std::min(kept, order.size());
    for (size_t k = 0; k < n; ++k) acc += w[order[k]];
    if (discarded) *discarded = 1.0 - acc;
  }
  std::vector<uint64_t> out(n);
  for (size_t k = 0; k < n; ++k) out[k] = strs[order[k]];
  return out;
}

// SinglesExtendHalfdets (extend.h:186-318): the strings and all their single
// excitations within norb orbitals, sorted, duplicates removed.
inline std::vector<uint64_t> SinglesExtend(const std::vector<uint64_t> &strs, int norb) {
  std::vector<uint64_t> out(strs);
  for (uint64_t v : strs)
    for (int i = 0; i < norb; ++i)
      if ((v >> i) & 1u)
        for (int a = 0; a < norb; ++a)
          if (!((v >> a) & 1u)) out.push_back(v ^ (1ull << i) ^ (1ull << a));
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return out;
}

// The carry-over branch of diag (sbdiag.h:749-796) for a solved problem.
inline void CarryOver(Problem &p, int norb, const std::vector<uint64_t> &adet, const std::vector<uint64_t> &bdet,
                      const std::vector<double> &W, int carryover_type, double ratio, double threshold,
                      std::vector<uint64_t> &co_adet, std::vector<uint64_t> &co_bdet) {
  if (carryover_type == 1 || carryover_type == 2) {
    std::vector<double> wa(adet.size()), wb(bdet.size());
    check(sbdgb_string_weights(p.get(), W.data(), wa.data(), wb.data(), nullptr), p.ctx(), "CarryOver");
    if (ratio == 0.0) {
      co_adet = carry_over_select(adet, wa, threshold, (size_t)-1, nullptr);
      co_bdet = carry_over_select(bdet, wb, threshold, (size_t)-1, nullptr);
    } else {
      double t = 0.0;
      co_adet = carry_over_select(adet, wa, 0.0, (size_t)(ratio * adet.size()), &t);
      co_bdet = carry_over_select(bdet, wb, 0.0, (size_t)(ratio * bdet.size()), &t);
    }
    if (carryover_type == 2) {
      co_adet = SinglesExtend(co_adet, norb);
      co_bdet = SinglesExtend(co_bdet, norb);
    }
  } else if (carryover_type == 3) {
    std::vector<uint64_t> ca(adet.size()), cb(bdet.size());
    double total = 0.0;
    check(sbdgb_string_cut_counts(p.get(), W.data(), threshold, ca.data(), cb.data(), &total, nullptr), p.ctx(),
          "CarryOver");
    std::vector<uint64_t> a, b;
    for (size_t i = 0; i < adet.size(); ++i)
      if (ca[i]) a.push_back(adet[i]);
    for (size_t i = 0; i < bdet.size(); ++i)
      if (cb[i]) b.push_back(bdet[i]);
    co_adet = SinglesExtend(a, norb);
    co_bdet = SinglesExtend(b, norb);
  } else {
    co_adet.clear();
    co_bdet.clear();
  }
}

// Device operator with the reference's MultBase::run shape (chemistry/basic/
// mult.h:19-103) over raw device pointers: Wb = hii o Wk + H_offdiag Wk.
class MultTPBGB300 {
 public:
  explicit MultTPBGB300(Problem &p) : p_(p) {
    check(sbdgb_diag_terms(p.get(), nullptr), p.ctx(), "MultTPBGB300 init");
  }
  // accumulate = true gives the reference's Wb += H Wk
  void run(const double *Wk_dev, double *Wb_dev, bool accumulate = true, void *stream = nullptr) {
    check(sbdgb_sigma(p_.get(), Wk_dev, Wb_dev, accumulate ? 1 : 0, stream), p_.ctx(), "MultTPBGB300::run");
  }
  int h_comm_size() const { return 1; }
  int b_comm_size() const { return 1; }
  int t_comm_size() const { return 1; }

 private:
  Problem &p_;
};

namespace tpb {

// Options of sbd::tpb::SBD (sbdiag.h:24-54) with the same defaults.
struct SBD {
  int task_comm_size = 1;
  int adet_comm_size = 1;
  int bdet_comm_size = 1;
  int h_comm_size = 1;
  int method = 0;
  int max_it = 1;
  int max_nb = 10;
  double eps = 1.0e-4;
  double max_time = 86400.0;
  int init = 0;
  size_t seed = 1729;
  int do_shuffle = 0;
  int do_rdm = 0;
  int carryover_type = 0;
  double ratio = 0.0;
  double threshold = 0.01;
  size_t bit_length = 20;
  // engine extensions
  int nroots = 1;
  int precision = SBDGB_FP64;
  int refine_every = 0;
  int device = 0;
};

// generate_sbd_data (sbdiag.h:56-134) for the flags this engine honours.
inline SBD generate_sbd_data(int argc, char *argv[]) {
  SBD d;
  for (int i = 0; i + 1 < argc; ++i) {
    const std::string a(argv[i]);
    const char *v = argv[i + 1];
    if (a == "--adet_comm_size") d.adet_comm_size = std::atoi(v);
    else if (a == "--bdet_comm_size") d.bdet_comm_size = std::atoi(v);
    else if (a == "--task_comm_size") d.task_comm_size = std::atoi(v);
    else if (a == "--method") d.method = std::atoi(v);
    else if (a == "--init") d.init = std::atoi(v);
    else if (a == "--seed") d.seed = std::atoi(v);
    else if (a == "--iteration") d.max_it = std::atoi(v);
    else if (a == "--block") d.max_nb = std::atoi(v);
    else if (a == "--tolerance") d.eps = std::atof(v);
    else if (a == "--max_time") d.max_time = std::atof(v);
    else if (a == "--rdm") d.do_rdm = std::atoi(v);
    else if (a == "--carryover_type") d.carryover_type = std::atoi(v);
    else if (a == "--carryover_ratio") d.ratio = std::atof(v);
    else if (a == "--carryover_threshold") d.threshold = std::atof(v);
    else if (a == "--bit_length") d.bit_length = std::atoi(v);
    else if (a == "--nroots") d.nroots = std::atoi(v);
    else if (a == "--precision") d.precision = std::atoi(v);
    else if (a == "--refine_every") d.refine_every = std::atoi(v);
    else if (a == "--device") d.device = std::atoi(v);
  }
  return d;
}

// diag (sbdiag.h:151-526) at communicator size 1: integrals -> tables ->
// diagonal -> Davidson (method 0 and 1) or Lanczos (method 2 and 3; the
// stored-Hamiltonian methods 1 and 3 give the same result matrix-free) ->
// energy.  Returns the ground energy in `energy`, the ground-state vector in
// *W and, with do_rdm == 0, the occupation density (sbdiag.h:666-699) in
// *density when those are non-null.  Carry-over strings, RDMs and wavefunction
// files are not produced by this entry point.
inline void diag(int comm_size, const SBD &sbd_data, const FCIDump &fcidump, const std::vector<uint64_t> &adet,
                 const std::vector<uint64_t> &bdet, double &energy, std::vector<double> *W = nullptr,
                 std::vector<double> *energies = nullptr, std::vector<double> *density = nullptr) {
  Context ctx(sbd_data.device);
  check(sbdgb_check_comm_sizes(ctx.get(), comm_size / std::max(1, sbd_data.task_comm_size * sbd_data.adet_comm_size *
                                                                      sbd_data.bdet_comm_size),
                               sbd_data.adet_comm_size * sbd_data.bdet_comm_size, sbd_data.task_comm_size),
        ctx.get(), "diag");
  if (sbd_data.method < 0 || sbd_data.method > 3) throw std::invalid_argument("--method must be 0..3");
  if (sbd_data.do_rdm != 0) throw std::invalid_argument("use the overload with RDM outputs for do_rdm != 0");
  const bool use_lanczos = (sbd_data.method & 2) != 0;
  Integrals ints = SetupIntegrals(fcidump);
  Problem p(ctx, ints, adet, bdet);
  sbdgb_davidson_opts o;
  sbdgb_davidson_default_opts(&o);
  o.max_it = sbd_data.max_it;
  o.max_nb = sbd_data.max_nb;
  o.eps = sbd_data.eps;
  o.max_time = sbd_data.max_time;
  o.nroots = sbd_data.nroots;
  o.init = sbd_data.init == 0 ? 0 : 1;
  o.precision = sbd_data.precision;
  o.refine_every = sbd_data.refine_every;
  if (use_lanczos) o.nroots = 1;
  std::vector<double> E(o.nroots), X;
  const bool want_x = W || density;
  if (want_x) X.resize(p.size() * o.nroots);
  sbdgb_report rep;
  if (use_lanczos)
    check(sbdgb_lanczos(p.get(), &o, E.data(), want_x ? X.data() : nullptr, &rep), ctx.get(), "diag");
  else
    check(sbdgb_davidson(p.get(), &o, E.data(), want_x ? X.data() : nullptr, &rep), ctx.get(), "diag");
  energy = E[0];
  if (energies) *energies = E;
  if (density) {
    density->assign(2 * (size_t)ints.L, 0.0);
    check(sbdgb_occupation_density(p.get(), X.data(), density->data(), nullptr), ctx.get(), "diag density");
  }
  if (W) W->assign(X.begin(), X.begin() + p.size());
}

// diag with the reference's argument list (sbdiag.h:151-163) at communicator
// size 1: loadname / savename name wavefunction files (LoadWavefunction gives
// the starting vector, SaveWavefunction stores the result); density is the
// occupation density (from the one-particle RDM when do_rdm != 0); co_adet /
// co_bdet are the carry-over strings of carryover_type 1..3; one_p_rdm /
// two_p_rdm are filled when do_rdm != 0.
inline void diag(int comm_size, const SBD &sbd_data, const FCIDump &fcidump, const std::vector<uint64_t> &adet,
                 const std::vector<uint64_t> &bdet, const std::string &loadname, const std::string &savename,
                 double &energy, std::vector<double> &density, std::vector<uint64_t> &co_adet,
                 std::vector<uint64_t> &co_bdet, std::vector<std::vector<double>> &one_p_rdm,
                 std::vector<std::vector<double>> &two_p_rdm) {
  Context ctx(sbd_data.device);
  check(sbdgb_check_comm_sizes(ctx.get(), comm_size / std::max(1, sbd_data.task_comm_size * sbd_data.adet_comm_size *
                                                                      sbd_data.bdet_comm_size),
                               sbd_data.adet_comm_size * sbd_data.bdet_comm_size, sbd_data.task_comm_size),
        ctx.get(), "diag");
  if (sbd_data.method < 0 || sbd_data.method > 3) throw std::invalid_argument("--method must be 0..3");
  const bool use_lanczos = (sbd_data.method & 2) != 0;
  Integrals ints = SetupIntegrals(fcidump);
  const int L = ints.L;
  Problem p(ctx, ints, adet, bdet);
  sbdgb_davidson_opts o;
  sbdgb_davidson_default_opts(&o);
  o.max_it = sbd_data.max_it;
  o.max_nb = sbd_data.max_nb;
  o.eps = sbd_data.eps;
  o.max_time = sbd_data.max_time;
  o.nroots = use_lanczos ? 1 : sbd_data.nroots;
  o.init = sbd_data.init == 0 ? 0 : 1;
  o.precision = sbd_data.precision;
  o.refine_every = sbd_data.refine_every;
  std::vector<double> E(o.nroots), X(p.size() * o.nroots);
  if (!loadname.empty()) {
    std::vector<double> W0;
    LoadWavefunction(loadname, adet, bdet, W0, sbd_data.bit_length);
    std::copy(W0.begin(), W0.end(), X.begin());
    o.init = 2;
    if (o.nroots > 1) throw std::invalid_argument("a loaded wavefunction starts one root");
  }
  sbdgb_report rep;
  if (use_lanczos)
    check(sbdgb_lanczos(p.get(), &o, E.data(), X.data(), &rep), ctx.get(), "diag");
  else
    check(sbdgb_davidson(p.get(), &o, E.data(), X.data(), &rep), ctx.get(), "diag");
  energy = E[0];
  std::vector<double> W(X.begin(), X.begin() + p.size());
  density.assign(2 * (size_t)L, 0.0);
  if (sbd_data.do_rdm == 0) {
    check(sbdgb_occupation_density(p.get(), W.data(), density.data(), nullptr), ctx.get(), "diag density");
  } else {
    Correlation(p, L, W, one_p_rdm, two_p_rdm);
    for (int io = 0; io < L; ++io) {
      density[2 * io] = one_p_rdm[0][io + (size_t)L * io];
      density[2 * io + 1] = one_p_rdm[1][io + (size_t)L * io];
    }
  }
  CarryOver(p, L, adet, bdet, W, sbd_data.carryover_type, sbd_data.ratio, sbd_data.threshold, co_adet, co_bdet);
  if (!savename.empty()) SaveWavefunction(savename, adet, bdet, L, W, sbd_data.bit_length);
}

}  // namespace tpb
}  // namespace sbdgb
