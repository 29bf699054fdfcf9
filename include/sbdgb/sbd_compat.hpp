// sbdgb/sbd_compat.hpp -- the reference's TPB entry points with the
// reference's own argument lists and types, over the GB300 engine.
//
// A caller written against the reference's namespace sbd (its app, or an SQD
// driver calling diag / MakeHelpers / makeQChamDiagTerms / mult / Davidson)
// compiles against this header unchanged once `sbd` names `sbdgb`
// (`namespace sbd = sbdgb;`).  The communicators are real MPI communicators
// (the caller's <mpi.h>, or any single-rank stand-in with the same names); the
// engine is one GPU per problem, so every communicator must have size 1 and
// every *_comm_size must be 1, or the call throws std::runtime_error.
//
// Reference interfaces mirrored (paths inside the reference project):
//   det_kind, det_vector<size_t, det_kind::half> .. framework/det_vector.h:42-818
//   LoadAlphaDets(file, dets, bit_length, L) ...... chemistry/basic/makedeterminants.h:167-191
//   sort_bitarray, makestring ...................... framework/bit_manipulation.h:195-233, 386-439
//   MpiBcast (FCIDump, det_vector) ................ framework/mpi_utility.h
//   oneInt, twoInt ................................ chemistry/basic/integrals.h:10-108
//   SetupIntegrals(fcidump, L, N, I0, I1, I2) ..... chemistry/basic/makeintegrals.h:123-174
//   TaskHelpers, MakeHelpers ...................... chemistry/tpb/helper.h:14-66, 729-873
//   makeQChamDiagTerms(adets, ..., hii, comms) .... chemistry/tpb/qcham.h:289-301
//   mult(hii, Wk, Wb, adets, ..., comms) .......... chemistry/tpb/mult.h:114-130
//   Davidson(hii, W, adets, ..., max_time) ........ chemistry/tpb/davidson.h:707-726
//   MultBase<ElemT>::run(hii, Wk, Wb) ............. chemistry/basic/mult.h:19-103
//   tpb::diag(comm, sbd_data, fcidump, adet, ...) . chemistry/tpb/sbdiag.h:151-163
//   tpb::diag(comm, sbd_data, fcidumpfile, ...) ... chemistry/tpb/sbdiag.h:846-857
//
// The engine state (device context, uploaded strings and integrals, tables)
// lives in the TaskHelpers that MakeHelpers returns and is reused by every call
// that receives them; a call with other integrals than the previous one
// re-uploads them (keyed on a hash of the integral values).
#pragma once

#include <mpi.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "sbdgb/tpb.hpp"

namespace sbdgb {

// ---- communicators -------------------------------------------------------------

inline void require_single_rank(MPI_Comm comm, const char *what) {
  int size = 1;
  MPI_Comm_size(comm, &size);
  if (size != 1)
    throw std::runtime_error(std::string(what) + ": communicator of size " + std::to_string(size) +
                             "; the GB300 engine solves a problem on one GPU (size 1)");
}

// ---- string tables -------------------------------------------------------------

enum class det_kind { full, half };

// Row-major table of strings, each row `width()` words of bit_length bits
// (word w holds orbitals [w*bit_length, (w+1)*bit_length)), as the reference's
// det_vector stores them.  Rows are views: a[i][w], a[i].size(), a[i].data().
template <typename ElemT, det_kind Kind = det_kind::full>
class det_vector {
 public:
  template <typename P>
  class row_view {
   public:
    row_view(P *p, size_t n) : p_(p), n_(n) {}
    P &operator[](size_t k) const { return p_[k]; }
    size_t size() const { return n_; }
    P *data() const { return p_; }
    P *begin() const { return p_; }
    P *end() const { return p_ + n_; }
    explicit operator std::vector<ElemT>() const { return std::vector<ElemT>(p_, p_ + n_); }

   private:
    P *p_;
    size_t n_;
  };

  det_vector() = default;
  det_vector(size_t n, size_t width) : data_(n * width, ElemT(0)), width_(width) {}

  size_t size() const { return width_ ? data_.size() / width_ : 0; }
  bool empty() const { return size() == 0; }
  size_t width() const { return width_; }
  void clear() { data_.clear(); }
  // Sets the row width of an empty table.
  void set_width(size_t w) {
    if (!data_.empty() && w != width_) throw std::length_error("det_vector: width of a non-empty table");
    width_ = w;
  }
  void resize(size_t n) { data_.resize(n * width_, ElemT(0)); }
  void push_back(const std::vector<ElemT> &r) {
    if (width_ == 0) width_ = r.size();
    if (r.size() != width_) throw std::length_error("det_vector::push_back: row width mismatch");
    data_.insert(data_.end(), r.begin(), r.end());
  }
  row_view<ElemT> operator[](size_t i) { return row_view<ElemT>(data_.data() + i * width_, width_); }
  row_view<const ElemT> operator[](size_t i) const { return row_view<const ElemT>(data_.data() + i * width_, width_); }
  ElemT *data() { return data_.data(); }
  const ElemT *data() const { return data_.data(); }

 private:
  std::vector<ElemT> data_;
  size_t width_ = 0;
};

using half_dets = det_vector<size_t, det_kind::half>;

// Words of bit_length bits -> one uint64 per string (norb <= 64).
inline uint64_t string_value(const size_t *w, size_t width, size_t bit_length) {
  uint64_t v = 0;
  for (size_t k = 0; k < width; ++k) v |= (uint64_t)w[k] << (k * bit_length);
  return v;
}
inline std::vector<size_t> string_words(uint64_t v, size_t width, size_t bit_length) {
  const uint64_t mask = bit_length >= 64 ? ~0ull : ((1ull << bit_length) - 1ull);
  std::vector<size_t> w(width);
  for (size_t k = 0; k < width; ++k) w[k] = (size_t)((v >> (k * bit_length)) & mask);
  return w;
}
inline std::vector<uint64_t> to_values(const half_dets &d, size_t bit_length) {
  std::vector<uint64_t> v(d.size());
  for (size_t i = 0; i < d.size(); ++i) v[i] = string_value(d[i].data(), d.width(), bit_length);
  return v;
}
inline half_dets from_values(const std::vector<uint64_t> &v, size_t bit_length, size_t L) {
  half_dets d;
  d.set_width((L + bit_length - 1) / bit_length);
  for (uint64_t x : v) d.push_back(string_words(x, d.width(), bit_length));
  return d;
}

// LoadAlphaDets(file, dets, bit_length, L): one string per line, orbital L-1
// first; appended in file order (sort_bitarray orders them).
inline void LoadAlphaDets(const std::string &file, half_dets &dets, size_t bit_length, size_t L) {
  if (L > 64) throw std::invalid_argument("norb > 64 is not supported");
  std::ifstream in(file);
  if (!in.is_open()) throw std::runtime_error("Failed to open alpha det file.");
  dets.clear();
  dets.set_width((L + bit_length - 1) / bit_length);
  std::string line;
  while (std::getline(in, line)) {
    if (line.empty()) continue;
    dets.push_back(string_words(from_string(line, (int)L), dets.width(), bit_length));
  }
}

// sort_bitarray: ascending with the last word most significant, duplicates
// removed (the string index order of every other call).
template <det_kind K>
inline void sort_bitarray(det_vector<size_t, K> &dets) {
  const size_t w = dets.width(), n = dets.size();
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) order[i] = i;
  auto less = [&](size_t x, size_t y) {
    for (size_t k = w; k > 0; --k) {
      if (dets[x][k - 1] != dets[y][k - 1]) return dets[x][k - 1] < dets[y][k - 1];
    }
    return false;
  };
  std::stable_sort(order.begin(), order.end(), less);
  det_vector<size_t, K> out;
  out.set_width(w);
  for (size_t i = 0; i < n; ++i) {
    if (i > 0 && !less(order[i - 1], order[i])) continue;
    out.push_back(std::vector<size_t>(dets[order[i]]));
  }
  dets = out;
}

// makestring(row, bit_length, L): orbital L-1 first, '1' = occupied.
template <typename Row>
inline std::string makestring(const Row &r, size_t bit_length, size_t L) {
  std::string s(L, '0');
  for (size_t i = 0; i < L; ++i)
    if ((r[i / bit_length] >> (i % bit_length)) & 1u) s[L - 1 - i] = '1';
  return s;
}

// ShuffleDet(dets, seed): a seeded permutation of the rows (std::mt19937).  The
// permutation is not the reference's; nothing computed here depends on the
// order of a list (diag orders the lists it is given).
template <det_kind K>
inline void ShuffleDet(det_vector<size_t, K> &dets, unsigned int seed) {
  std::vector<size_t> order(dets.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::mt19937 g(seed);
  std::shuffle(order.begin(), order.end(), g);
  det_vector<size_t, K> out;
  out.set_width(dets.width());
  for (size_t i : order) out.push_back(std::vector<size_t>(dets[i]));
  dets = out;
}

// Broadcasts of the reference app: nothing moves at communicator size 1.
template <typename T>
inline void MpiBcast(T &, int root, MPI_Comm comm) {
  require_single_rank(comm, "MpiBcast");
  if (root != 0) throw std::invalid_argument("MpiBcast: root must be rank 0");
}

// ---- integrals -----------------------------------------------------------------

// One-body integrals over 2L spin orbitals, row-major (alpha p -> 2p, beta p -> 2p+1).
template <typename ElemT>
class oneInt {
 public:
  std::vector<ElemT> store;
  int norbs = 0;
  ElemT &operator()(int i, int j) { return store.at((size_t)i * norbs + j); }
  ElemT Value(int i, int j) const { return store.at((size_t)i * norbs + j); }
};

// Two-body integrals: spatial (IJ|KL), 8-fold packed, addressed with
// spin-orbital indices (zero unless spin(i) = spin(j) and spin(k) = spin(l));
// Direct/Exchange tables over 2L spin orbitals, column-major.
template <typename ElemT>
class twoInt {
 public:
  std::vector<ElemT> store;
  ElemT maxEntry = ElemT(100.0);
  ElemT zero = ElemT(0.0);
  int norbs = 0;
  std::vector<ElemT> DirectMat, ExchangeMat;
  static size_t index(int i, int j, int k, int l) {
    const size_t ij = pair_index(i / 2, j / 2), kl = pair_index(k / 2, l / 2);
    const size_t a = std::max(ij, kl), b = std::min(ij, kl);
    return a * (a + 1) / 2 + b;
  }
  ElemT &operator()(int i, int j, int k, int l) {
    zero = ElemT(0.0);
    if (!((i % 2 == j % 2) && (k % 2 == l % 2))) return zero;
    return store[index(i, j, k, l)];
  }
  ElemT Value(int i, int j, int k, int l) const {
    if (!((i % 2 == j % 2) && (k % 2 == l % 2))) return ElemT(0.0);
    return store[index(i, j, k, l)];
  }
  ElemT &Direct(int i, int j) { return DirectMat[(size_t)i + 2 * (size_t)norbs * j]; }
  ElemT &Exchange(int i, int j) { return ExchangeMat[(size_t)i + 2 * (size_t)norbs * j]; }
  ElemT DirectValue(int i, int j) const { return DirectMat[(size_t)i + 2 * (size_t)norbs * j]; }
  ElemT ExchangeValue(int i, int j) const { return ExchangeMat[(size_t)i + 2 * (size_t)norbs * j]; }
};

// SetupIntegrals(fcidump, L, N, I0, I1, I2): the same values in the
// reference's layouts, from the engine's own FCIDUMP reader.
template <typename ElemT>
inline void SetupIntegrals(const FCIDump &fcidump, int &L, int &N, ElemT &I0, oneInt<ElemT> &I1, twoInt<ElemT> &I2) {
  const Integrals t = SetupIntegrals(fcidump);
  L = t.L;
  N = t.N;
  I0 = ElemT(t.I0);
  I1.norbs = 2 * L;
  I1.store.assign((size_t)4 * L * L, ElemT(0.0));
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < L; ++j) {
      I1(2 * i, 2 * j) = ElemT(t.h1[(size_t)i * L + j]);
      I1(2 * i + 1, 2 * j + 1) = ElemT(t.h1[(size_t)i * L + j]);
    }
  I2.norbs = L;
  I2.store.assign(t.eri.begin(), t.eri.end());
  I2.DirectMat.assign((size_t)4 * L * L, ElemT(0.0));
  I2.ExchangeMat.assign((size_t)4 * L * L, ElemT(0.0));
  for (int i = 0; i < 2 * L; ++i)
    for (int j = 0; j < 2 * L; ++j) {
      I2.Direct(i, j) = I2.Value(i, i, j, j);
      I2.Exchange(i, j) = I2.Value(i, j, j, i);
    }
}

namespace detail {

// Spatial h1 (L x L) and the packed ERI of the engine from the reference layouts.
template <typename ElemT>
inline Integrals engine_integrals(const ElemT &I0, const oneInt<ElemT> &I1, const twoInt<ElemT> &I2) {
  Integrals t;
  t.L = I2.norbs;
  t.I0 = (double)I0;
  if (I1.norbs != 2 * t.L) throw std::invalid_argument("oneInt and twoInt disagree on the orbital count");
  t.h1.resize((size_t)t.L * t.L);
  for (int i = 0; i < t.L; ++i)
    for (int j = 0; j < t.L; ++j) t.h1[(size_t)i * t.L + j] = (double)I1.Value(2 * i, 2 * j);
  t.eri.assign(I2.store.begin(), I2.store.end());
  return t;
}

inline uint64_t hash_bytes(uint64_t h, const void *p, size_t n) {
  const unsigned char *b = (const unsigned char *)p;
  for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
  return h;
}

// The engine objects behind one TaskHelpers: a context, the strings and the
// problem built for the integrals seen last.
struct EngineState {
  std::unique_ptr<Context> ctx;
  std::vector<uint64_t> astr, bstr;
  size_t bit_length = 20;
  int norb = 0;
  uint64_t ints_key = 0;
  std::unique_ptr<Problem> problem;

  template <typename ElemT>
  Problem &problem_for(const ElemT &I0, const oneInt<ElemT> &I1, const twoInt<ElemT> &I2) {
    uint64_t h = 14695981039346656037ull;
    const double i0 = (double)I0;
    h = hash_bytes(h, &i0, sizeof(i0));
    h = hash_bytes(h, I1.store.data(), I1.store.size() * sizeof(ElemT));
    h = hash_bytes(h, I2.store.data(), I2.store.size() * sizeof(ElemT));
    if (!problem || h != ints_key) {
      problem.reset();
      const Integrals t = engine_integrals(I0, I1, I2);
      if (t.L != norb) throw std::invalid_argument("integrals and helpers disagree on norb");
      problem.reset(new Problem(*ctx, t, astr, bstr));
      check(sbdgb_build_tables(problem->get()), ctx->get(), "MakeHelpers");
      ints_key = h;
    }
    return *problem;
  }
};

}  // namespace detail

// ---- helpers (chemistry/tpb/helper.h) --------------------------------------------

// The excitation lists of the whole problem as one task, in the reference's
// flat layout (CSR over bra strings, kets ascending, spin-orbital CrAn), plus
// the engine state the other calls use.
struct TaskHelpers {
  size_t braAlphaStart = 0, braAlphaEnd = 0, ketAlphaStart = 0, ketAlphaEnd = 0;
  size_t braBetaStart = 0, braBetaEnd = 0, ketBetaStart = 0, ketBetaEnd = 0;
  size_t taskType = 0, adetShift = 0, bdetShift = 0;
  std::vector<size_t> SinglesFromAlphaOffset, DoublesFromAlphaOffset, SinglesFromBetaOffset, DoublesFromBetaOffset;
  std::vector<size_t> SinglesFromAlpha_flat, DoublesFromAlpha_flat, SinglesFromBeta_flat, DoublesFromBeta_flat;
  std::vector<int> SinglesAlphaCrAn_flat, DoublesAlphaCrAn_flat, SinglesBetaCrAn_flat, DoublesBetaCrAn_flat;
  std::shared_ptr<detail::EngineState> engine;
};

inline std::shared_ptr<detail::EngineState> engine_of(const std::vector<TaskHelpers> &helper) {
  if (helper.empty() || !helper[0].engine) throw std::invalid_argument("helpers were not made by MakeHelpers");
  return helper[0].engine;
}

// MakeHelpers(adets, bdets, bit_length, norb, helper, h_comm, b_comm, t_comm,
// adet_comm_size, bdet_comm_size): the excitation tables, built on the GPU.
// The lists must be sorted (sort_bitarray), as the reference's are.
inline void MakeHelpers(const half_dets &adets, const half_dets &bdets, size_t bit_length, size_t norb,
                        std::vector<TaskHelpers> &helper, MPI_Comm h_comm, MPI_Comm b_comm, MPI_Comm t_comm,
                        size_t adet_comm_size, size_t bdet_comm_size) {
  require_single_rank(h_comm, "MakeHelpers");
  require_single_rank(b_comm, "MakeHelpers");
  require_single_rank(t_comm, "MakeHelpers");
  if (adet_comm_size != 1 || bdet_comm_size != 1)
    throw std::runtime_error("MakeHelpers: adet/bdet communicator sizes must be 1 on the GB300 engine");
  auto st = std::make_shared<detail::EngineState>();
  int dev = 0;
  if (const char *e = std::getenv("SBDGB_DEVICE")) dev = std::atoi(e);
  st->ctx.reset(new Context(dev));
  st->bit_length = bit_length;
  st->norb = (int)norb;
  st->astr = to_values(adets, bit_length);
  st->bstr = to_values(bdets, bit_length);
  // the tables do not depend on the integrals: build them on a problem with zero integrals
  Integrals zero;
  zero.L = (int)norb;
  const size_t B = norb * (norb + 1) / 2;
  zero.h1.assign(norb * norb, 0.0);
  zero.eri.assign(B * (B + 1) / 2, 0.0);
  Problem p(*st->ctx, zero, st->astr, st->bstr);
  check(sbdgb_build_tables(p.get()), st->ctx->get(), "MakeHelpers");
  TaskHelpers t;
  t.braAlphaEnd = t.ketAlphaEnd = adets.size();
  t.braBetaEnd = t.ketBetaEnd = bdets.size();
  for (int spin = 0; spin < 2; ++spin) {
    uint64_t ns = 0, nd = 0;
    check(sbdgb_table_counts(p.get(), spin, &ns, &nd), st->ctx->get(), "MakeHelpers");
    const size_t n = spin == 0 ? adets.size() : bdets.size();
    std::vector<uint64_t> os(n + 1), ks(ns), od(n + 1), kd(nd);
    std::vector<int32_t> cs(2 * ns), cd(4 * nd);
    check(sbdgb_export_tables(p.get(), spin, os.data(), ks.data(), cs.data(), od.data(), kd.data(), cd.data()),
          st->ctx->get(), "MakeHelpers");
    (spin == 0 ? t.SinglesFromAlphaOffset : t.SinglesFromBetaOffset).assign(os.begin(), os.end());
    (spin == 0 ? t.DoublesFromAlphaOffset : t.DoublesFromBetaOffset).assign(od.begin(), od.end());
    (spin == 0 ? t.SinglesFromAlpha_flat : t.SinglesFromBeta_flat).assign(ks.begin(), ks.end());
    (spin == 0 ? t.DoublesFromAlpha_flat : t.DoublesFromBeta_flat).assign(kd.begin(), kd.end());
    (spin == 0 ? t.SinglesAlphaCrAn_flat : t.SinglesBetaCrAn_flat).assign(cs.begin(), cs.end());
    (spin == 0 ? t.DoublesAlphaCrAn_flat : t.DoublesBetaCrAn_flat).assign(cd.begin(), cd.end());
  }
  t.engine = st;
  helper.assign(1, t);
}

// ---- operator calls ------------------------------------------------------------

// makeQChamDiagTerms(adets, bdets, bit_length, norbs, helper, I0, I1, I2, hii, comms).
template <typename ElemT>
inline void makeQChamDiagTerms(const half_dets &adets, const half_dets &bdets, const size_t bit_length,
                               const size_t norbs, const std::vector<TaskHelpers> &helper, ElemT &I0,
                               oneInt<ElemT> &I1, twoInt<ElemT> &I2, std::vector<ElemT> &hii, MPI_Comm h_comm,
                               MPI_Comm b_comm, MPI_Comm t_comm) {
  static_assert(std::is_same<ElemT, double>::value, "the GB300 engine computes in double");
  require_single_rank(h_comm, "makeQChamDiagTerms");
  require_single_rank(b_comm, "makeQChamDiagTerms");
  require_single_rank(t_comm, "makeQChamDiagTerms");
  auto st = engine_of(helper);
  if (adets.size() != st->astr.size() || bdets.size() != st->bstr.size() || norbs != (size_t)st->norb ||
      bit_length != st->bit_length)
    throw std::invalid_argument("makeQChamDiagTerms: strings differ from the helpers'");
  Problem &p = st->problem_for(I0, I1, I2);
  hii.resize(p.size());
  check(sbdgb_diag_terms(p.get(), hii.data()), p.ctx(), "makeQChamDiagTerms");
}

// mult(hii, Wk, Wb, adets, bdets, bit_length, norbs, adet_comm_size,
// bdet_comm_size, helper, I0, I1, I2, h_comm, b_comm, t_comm): Wb += H Wk,
// with hii as the diagonal.
template <typename ElemT>
inline void mult(const std::vector<ElemT> &hii, const std::vector<ElemT> &Wk, std::vector<ElemT> &Wb,
                 const half_dets &adets, const half_dets &bdets, const size_t bit_length, const size_t norbs,
                 const size_t adet_comm_size, const size_t bdet_comm_size, const std::vector<TaskHelpers> &helper,
                 const ElemT &I0, const oneInt<ElemT> &I1, const twoInt<ElemT> &I2, MPI_Comm h_comm, MPI_Comm b_comm,
                 MPI_Comm t_comm) {
  static_assert(std::is_same<ElemT, double>::value, "the GB300 engine computes in double");
  require_single_rank(h_comm, "mult");
  require_single_rank(b_comm, "mult");
  require_single_rank(t_comm, "mult");
  if (adet_comm_size != 1 || bdet_comm_size != 1) throw std::runtime_error("mult: communicator sizes must be 1");
  auto st = engine_of(helper);
  if (adets.size() != st->astr.size() || bdets.size() != st->bstr.size() || norbs != (size_t)st->norb ||
      bit_length != st->bit_length)
    throw std::invalid_argument("mult: strings differ from the helpers'");
  Problem &p = st->problem_for(I0, I1, I2);
  if (Wk.size() != p.size() || Wb.size() != p.size() || (hii.size() != p.size() && !hii.empty()))
    throw std::invalid_argument("mult: vector size mismatch");
  check(sbdgb_mult_host(p.get(), hii.empty() ? nullptr : hii.data(), Wk.data(), Wb.data()), p.ctx(), "mult");
}

// Davidson(hii, W, adets, bdets, bit_length, norbs, adet_comm_size,
// bdet_comm_size, helper, I0, I1, I2, h_comm, b_comm, t_comm, max_iteration,
// num_block, eps, max_time): W in = starting vector, out = the normalised
// ground-state vector (one root, FP64, the engine's Davidson).
template <typename ElemT, typename RealT>
inline void Davidson(const std::vector<ElemT> &hii, std::vector<ElemT> &W, const half_dets &adets,
                     const half_dets &bdets, const size_t bit_length, const size_t norbs, const size_t adet_comm_size,
                     const size_t bdet_comm_size, const std::vector<TaskHelpers> &helper, const ElemT &I0,
                     const oneInt<ElemT> &I1, const twoInt<ElemT> &I2, MPI_Comm h_comm, MPI_Comm b_comm,
                     MPI_Comm t_comm, int max_iteration, int num_block, RealT eps, RealT max_time) {
  static_assert(std::is_same<ElemT, double>::value, "the GB300 engine computes in double");
  require_single_rank(h_comm, "Davidson");
  require_single_rank(b_comm, "Davidson");
  require_single_rank(t_comm, "Davidson");
  if (adet_comm_size != 1 || bdet_comm_size != 1) throw std::runtime_error("Davidson: communicator sizes must be 1");
  (void)hii;  // the engine's diagonal is the same hii (makeQChamDiagTerms)
  auto st = engine_of(helper);
  if (adets.size() != st->astr.size() || bdets.size() != st->bstr.size() || norbs != (size_t)st->norb ||
      bit_length != st->bit_length)
    throw std::invalid_argument("Davidson: strings differ from the helpers'");
  Problem &p = st->problem_for(I0, I1, I2);
  sbdgb::Davidson(p, W, max_iteration, num_block, (double)eps, (double)max_time, W.size() == p.size() ? 2 : 0);
}

// ---- operator plugin (chemistry/basic/mult.h) ------------------------------------

// The reference's operator interface: run(hii, Wk, Wb) computes Wb += H Wk.
template <typename ElemT>
class MultBase {
 public:
  MultBase() = default;
  MultBase(uint32_t bit_length, size_t norbs, MPI_Comm h_comm, MPI_Comm b_comm, MPI_Comm t_comm)
      : bit_length_(bit_length), norbs_(norbs), h_comm_(h_comm), b_comm_(b_comm), t_comm_(t_comm) {
    D_size_ = (2 * norbs + bit_length - 1) / bit_length;
  }
  virtual ~MultBase() = default;
  uint32_t bit_length() const { return bit_length_; }
  size_t norbs() const { return norbs_; }
  size_t D_size() const { return D_size_; }
  MPI_Comm h_comm() const { return h_comm_; }
  MPI_Comm b_comm() const { return b_comm_; }
  MPI_Comm t_comm() const { return t_comm_; }
  MPI_Comm a_comm() const { return MPI_COMM_SELF; }
  virtual void run(const std::vector<ElemT> &hii, const std::vector<ElemT> &Wk, std::vector<ElemT> &Wb) = 0;

 protected:
  uint32_t bit_length_ = 20;
  size_t norbs_ = 0, D_size_ = 0;
  MPI_Comm h_comm_ = MPI_COMM_SELF, b_comm_ = MPI_COMM_SELF, t_comm_ = MPI_COMM_SELF;
};

// MultBase over the GB300 engine: construction uploads strings and integrals
// and builds the tables; run() is mult() on host vectors, run_device() the same
// product on device pointers (N doubles each, accumulate or overwrite).
template <typename ElemT>
class MultTPB : public MultBase<ElemT> {
 public:
  MultTPB(const half_dets &adets, const half_dets &bdets, size_t bit_length, size_t norbs,
          const std::vector<TaskHelpers> &helper, const ElemT &I0, const oneInt<ElemT> &I1, const twoInt<ElemT> &I2,
          MPI_Comm h_comm, MPI_Comm b_comm, MPI_Comm t_comm)
      : MultBase<ElemT>((uint32_t)bit_length, norbs, h_comm, b_comm, t_comm), engine_(engine_of(helper)) {
    static_assert(std::is_same<ElemT, double>::value, "the GB300 engine computes in double");
    require_single_rank(h_comm, "MultTPB");
    require_single_rank(b_comm, "MultTPB");
    require_single_rank(t_comm, "MultTPB");
    if (adets.size() != engine_->astr.size() || bdets.size() != engine_->bstr.size())
      throw std::invalid_argument("MultTPB: strings differ from the helpers'");
    problem_ = &engine_->problem_for(I0, I1, I2);
    check(sbdgb_diag_terms(problem_->get(), nullptr), problem_->ctx(), "MultTPB");
  }
  void run(const std::vector<ElemT> &hii, const std::vector<ElemT> &Wk, std::vector<ElemT> &Wb) override {
    if (Wk.size() != problem_->size() || Wb.size() != problem_->size())
      throw std::invalid_argument("MultTPB::run: vector size mismatch");
    check(sbdgb_mult_host(problem_->get(), hii.empty() ? nullptr : hii.data(), Wk.data(), Wb.data()),
          problem_->ctx(), "MultTPB::run");
  }
  void run_device(const ElemT *Wk_dev, ElemT *Wb_dev, bool accumulate = true, void *stream = nullptr) {
    check(sbdgb_sigma(problem_->get(), Wk_dev, Wb_dev, accumulate ? 1 : 0, stream), problem_->ctx(),
          "MultTPB::run_device");
  }
  Problem &problem() { return *problem_; }

 private:
  std::shared_ptr<detail::EngineState> engine_;
  Problem *problem_ = nullptr;
};

namespace tpb {

// diag(comm, sbd_data, fcidump, adet, bdet, loadname, savename, energy,
// density, co_adet, co_bdet, one_p_rdm, two_p_rdm) with the reference's types.
// Lists in any order are accepted (they are ordered here, as sort_bitarray
// would); the outputs do not depend on the order.
inline void diag(const MPI_Comm &comm, const SBD &sbd_data, const FCIDump &fcidump, const half_dets &adet,
                 const half_dets &bdet, const std::string &loadname, const std::string &savename, double &energy,
                 std::vector<double> &density, half_dets &co_adet, half_dets &co_bdet,
                 std::vector<std::vector<double>> &one_p_rdm, std::vector<std::vector<double>> &two_p_rdm) {
  require_single_rank(comm, "diag");
  int L = 0;
  for (const auto &kv : fcidump.header)
    if (kv.first == "NORB") L = std::atoi(kv.second.c_str());
  std::vector<uint64_t> a = to_values(adet, sbd_data.bit_length), b = to_values(bdet, sbd_data.bit_length);
  std::sort(a.begin(), a.end());
  a.erase(std::unique(a.begin(), a.end()), a.end());
  std::sort(b.begin(), b.end());
  b.erase(std::unique(b.begin(), b.end()), b.end());
  std::vector<uint64_t> ca, cb;
  diag(1, sbd_data, fcidump, a, b, loadname, savename, energy, density, ca, cb, one_p_rdm, two_p_rdm);
  co_adet = from_values(ca, sbd_data.bit_length, (size_t)L);
  co_bdet = from_values(cb, sbd_data.bit_length, (size_t)L);
}

// diag(comm, sbd_data, fcidumpfile, adetfile, ...): the file-name form; the
// beta list is the alpha list.
inline void diag(const MPI_Comm &comm, const SBD &sbd_data, const std::string &fcidumpfile,
                 const std::string &adetfile, const std::string &loadname, const std::string &savename,
                 double &energy, std::vector<double> &density, half_dets &co_adet, half_dets &co_bdet,
                 std::vector<std::vector<double>> &one_p_rdm, std::vector<std::vector<double>> &two_p_rdm) {
  require_single_rank(comm, "diag");
  const FCIDump fcidump = LoadFCIDump(fcidumpfile);
  int L = 0;
  for (const auto &kv : fcidump.header)
    if (kv.first == "NORB") L = std::atoi(kv.second.c_str());
  half_dets adet;
  LoadAlphaDets(adetfile, adet, sbd_data.bit_length, (size_t)L);
  sort_bitarray(adet);
  diag(comm, sbd_data, fcidump, adet, adet, loadname, savename, energy, density, co_adet, co_bdet, one_p_rdm,
       two_p_rdm);
}

}  // namespace tpb
}  // namespace sbdgb
