// Reference harness: drives the reference's own header-only TPB CPU path
// (SBD_TRADMODE, OpenMP, MPI size 1) on FCIDUMP + string files and writes
// its intermediate results in a small tagged binary format.
//
// Test infrastructure only.  Built by oracle/Makefile into oracle/_ref/ from
// the reference headers where they lie; used to pin the C restatement and to
// generate the golden fixtures under tests/golden/.  Nothing in the product
// library links or calls it.
//
// Flow mirrors sbd::tpb::diag (chemistry/tpb/sbdiag.h:151-526):
//   SetupIntegrals -> TaskCommunicator -> MakeHelpers -> RemakeHelpers ->
//   BasisInitVector(init 0) -> makeQChamDiagTerms -> Davidson(max_time) ->
//   final mult and <W|HW>.
//
// Usage:
//   sbdref --fcidump F --adet A [--bdet B] --out OUTFILE
//          [--bit_length 20] [--tables 1] [--hii 1] [--cvec C.bin]
//          [--davidson 1 --block NB --iteration IT --tolerance EPS]
//          [--time_mult K] [--density 1] [--rdm 1]
//          [--lanczos 1 --lanczos_block NB --lanczos_iteration IT --lanczos_tolerance EPS]
//          [--save NAME] [--load NAME]
//          [--carryover TYPE --carryover_ratio R --carryover_threshold T]
// --carryover runs the carry-over branch of sbd::tpb::diag (chemistry/tpb/
// sbdiag.h:749-796) on the Davidson vector and outputs the selected strings.
// --save writes the Davidson vector with SaveWavefunction (chemistry/tpb/
// restart.h:21-67, file NAME000000); --load maps a saved wavefunction onto the
// current strings with LoadWavefunction (restart.h:415-660) and outputs it.
// --density and --rdm evaluate OccupationDensity (chemistry/tpb/occupation.h)
// and Correlation (chemistry/tpb/correlation.h) on the --cvec vector; --lanczos
// runs the matrix-free Lanczos (chemistry/tpb/lanczos.h:169) from the init-0
// vector, as sbd::tpb::diag does for --method 2.
#include <numeric>
#include <omp.h>
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "sbd/sbd.h"

namespace {

struct Out {
  std::ofstream f;
  explicit Out(const std::string &path) : f(path, std::ios::binary) {
    if (!f) throw std::runtime_error("cannot open output " + path);
  }
  // record: u32 name length, name bytes, u8 dtype code, u64 count, payload
  template <typename T>
  void put(const std::string &name, char code, const T *data, size_t n) {
    uint32_t len = (uint32_t)name.size();
    f.write((const char *)&len, 4);
    f.write(name.data(), len);
    f.write(&code, 1);
    uint64_t cnt = n;
    f.write((const char *)&cnt, 8);
    if (n) f.write((const char *)data, (std::streamsize)(n * sizeof(T)));
  }
  void u64(const std::string &name, const std::vector<size_t> &v) { put(name, 'Q', v.data(), v.size()); }
  void i32(const std::string &name, const std::vector<int> &v) { put(name, 'i', v.data(), v.size()); }
  void f64(const std::string &name, const std::vector<double> &v) { put(name, 'd', v.data(), v.size()); }
  void scalar(const std::string &name, double x) { put(name, 'd', &x, 1); }
};

std::string arg(int argc, char **argv, const char *key, const char *dflt) {
  for (int i = 1; i + 1 < argc; ++i)
    if (std::string(argv[i]) == key) return argv[i + 1];
  return dflt;
}

}  // namespace

int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  MPI_Comm comm = MPI_COMM_WORLD;
  const std::string fcifile = arg(argc, argv, "--fcidump", "");
  const std::string afile = arg(argc, argv, "--adet", "");
  const std::string bfile = arg(argc, argv, "--bdet", "");
  const std::string outfile = arg(argc, argv, "--out", "sbdref.bin");
  const std::string cfile = arg(argc, argv, "--cvec", "");
  const size_t bit_length = std::stoul(arg(argc, argv, "--bit_length", "20"));
  const int want_tables = std::stoi(arg(argc, argv, "--tables", "1"));
  const int want_hii = std::stoi(arg(argc, argv, "--hii", "1"));
  const int want_dav = std::stoi(arg(argc, argv, "--davidson", "0"));
  const int max_nb = std::stoi(arg(argc, argv, "--block", "10"));
  const int max_it = std::stoi(arg(argc, argv, "--iteration", "1"));
  const double eps = std::stod(arg(argc, argv, "--tolerance", "1e-4"));
  const int time_mult = std::stoi(arg(argc, argv, "--time_mult", "0"));
  const int want_density = std::stoi(arg(argc, argv, "--density", "0"));
  const int want_rdm = std::stoi(arg(argc, argv, "--rdm", "0"));
  const int want_lanczos = std::stoi(arg(argc, argv, "--lanczos", "0"));
  const std::string savename = arg(argc, argv, "--save", "");
  const int co_type = std::stoi(arg(argc, argv, "--carryover", "0"));
  const double co_ratio = std::stod(arg(argc, argv, "--carryover_ratio", "0"));
  const double co_threshold = std::stod(arg(argc, argv, "--carryover_threshold", "0.01"));
  const std::string loadname = arg(argc, argv, "--load", "");
  const int lz_nb = std::stoi(arg(argc, argv, "--lanczos_block", "40"));
  const int lz_it = std::stoi(arg(argc, argv, "--lanczos_iteration", "20"));
  const double lz_eps = std::stod(arg(argc, argv, "--lanczos_tolerance", "1e-12"));

  sbd::FCIDump fcidump = sbd::LoadFCIDump(fcifile);
  int L = 0, Ne = 0;
  double I0 = 0.0;
  sbd::oneInt<double> I1;
  sbd::twoInt<double> I2;
  sbd::SetupIntegrals(fcidump, L, Ne, I0, I1, I2);
  sbd::det_vector<size_t>::init_elem_size((2 * L + bit_length - 1) / bit_length);
  sbd::det_vector<size_t, sbd::det_kind::half>::init_elem_size((L + bit_length - 1) / bit_length);

  sbd::det_vector<size_t, sbd::det_kind::half> adet, bdet;
  sbd::LoadAlphaDets(afile, adet, bit_length, L);
  sbd::sort_bitarray(adet);
  if (bfile.empty()) {
    bdet = adet;
  } else {
    sbd::LoadAlphaDets(bfile, bdet, bit_length, L);
    sbd::sort_bitarray(bdet);
  }

  MPI_Comm h_comm, b_comm, t_comm, a_comm;
  sbd::TaskCommunicator(comm, 1, 1, 1, 1, h_comm, b_comm, t_comm, a_comm);
  std::vector<sbd::TaskHelpers> helper;
  auto th0 = std::chrono::steady_clock::now();
  sbd::MakeHelpers(adet, bdet, bit_length, L, helper, h_comm, b_comm, t_comm, 1, 1);
  sbd::RemakeHelpers(adet, bdet, bit_length, L, helper, h_comm, b_comm, t_comm, 1, 1);
  auto th1 = std::chrono::steady_clock::now();

  Out out(outfile);
  out.scalar("norb", (double)L);
  out.scalar("nalpha_str", (double)adet.size());
  out.scalar("nbeta_str", (double)bdet.size());
  out.scalar("threads", (double)omp_get_max_threads());
  out.scalar("t_helpers", std::chrono::duration<double>(th1 - th0).count());
  {
    // sorted strings, first word only when a string fits in one word
    std::vector<size_t> a(adet.size() * adet.elem_size()), b(bdet.size() * bdet.elem_size());
    for (size_t i = 0; i < adet.size(); ++i)
      for (size_t w = 0; w < adet.elem_size(); ++w) a[i * adet.elem_size() + w] = adet[i][w];
    for (size_t i = 0; i < bdet.size(); ++i)
      for (size_t w = 0; w < bdet.elem_size(); ++w) b[i * bdet.elem_size() + w] = bdet[i][w];
    out.u64("adet_words", a);
    out.u64("bdet_words", b);
  }

  if (want_tables) {
    for (size_t t = 0; t < helper.size(); ++t) {
      const auto &h = helper[t];
      std::string p = "task" + std::to_string(t) + ".";
      out.scalar(p + "type", (double)h.taskType);
      out.u64(p + "SinglesFromAlphaOffset", h.SinglesFromAlphaOffset);
      out.u64(p + "SinglesFromAlpha", h.SinglesFromAlpha_flat);
      out.i32(p + "SinglesAlphaCrAn", h.SinglesAlphaCrAn_flat);
      out.u64(p + "DoublesFromAlphaOffset", h.DoublesFromAlphaOffset);
      out.u64(p + "DoublesFromAlpha", h.DoublesFromAlpha_flat);
      out.i32(p + "DoublesAlphaCrAn", h.DoublesAlphaCrAn_flat);
      out.u64(p + "SinglesFromBetaOffset", h.SinglesFromBetaOffset);
      out.u64(p + "SinglesFromBeta", h.SinglesFromBeta_flat);
      out.i32(p + "SinglesBetaCrAn", h.SinglesBetaCrAn_flat);
      out.u64(p + "DoublesFromBetaOffset", h.DoublesFromBetaOffset);
      out.u64(p + "DoublesFromBeta", h.DoublesFromBeta_flat);
      out.i32(p + "DoublesBetaCrAn", h.DoublesBetaCrAn_flat);
    }
  }

  std::vector<double> hii;
  auto tq0 = std::chrono::steady_clock::now();
  sbd::makeQChamDiagTerms(adet, bdet, bit_length, L, helper, I0, I1, I2, hii, h_comm, b_comm, t_comm);
  auto tq1 = std::chrono::steady_clock::now();
  out.scalar("t_hii", std::chrono::duration<double>(tq1 - tq0).count());
  if (want_hii) out.f64("hii", hii);

  if (!cfile.empty()) {
    std::ifstream cf(cfile, std::ios::binary);
    std::vector<double> C(hii.size());
    cf.read((char *)C.data(), (std::streamsize)(C.size() * sizeof(double)));
    if (!cf) throw std::runtime_error("short C vector file");
    std::vector<double> S(C.size(), 0.0);
    auto tm0 = std::chrono::steady_clock::now();
    sbd::mult(hii, C, S, adet, bdet, bit_length, (size_t)L, 1, 1, helper, I0, I1, I2, h_comm, b_comm, t_comm);
    auto tm1 = std::chrono::steady_clock::now();
    out.scalar("t_mult", std::chrono::duration<double>(tm1 - tm0).count());
    out.f64("sigma", S);
    for (int k = 1; k < time_mult; ++k) {
      std::fill(S.begin(), S.end(), 0.0);
      auto a0 = std::chrono::steady_clock::now();
      sbd::mult(hii, C, S, adet, bdet, bit_length, (size_t)L, 1, 1, helper, I0, I1, I2, h_comm, b_comm, t_comm);
      auto a1 = std::chrono::steady_clock::now();
      out.scalar("t_mult", std::chrono::duration<double>(a1 - a0).count());
    }
    if (want_density) {
      std::vector<int> oIdx(L);
      std::iota(oIdx.begin(), oIdx.end(), 0);
      std::vector<double> res;
      sbd::OccupationDensity(oIdx, C, adet, bdet, bit_length, 1, 1, b_comm, res);
      out.f64("density_c", res);
    }
    if (want_rdm) {
      std::vector<std::vector<double>> one, two;
      sbd::Correlation(C, adet, bdet, bit_length, (size_t)L, 1, 1, helper, h_comm, b_comm, t_comm, one, two);
      for (int k = 0; k < 2; ++k) out.f64("rdm1_" + std::to_string(k), one[k]);
      for (int k = 0; k < 4; ++k) out.f64("rdm2_" + std::to_string(k), two[k]);
    }
  }

  if (want_lanczos) {
    std::vector<double> W;
    sbd::BasisInitVector(W, adet, bdet, 1, 1, h_comm, b_comm, t_comm, 0, 1729);
    sbd::Lanczos(hii, W, adet, bdet, bit_length, (size_t)L, 1, 1, helper, I0, I1, I2, h_comm, b_comm, t_comm,
                 lz_it, lz_nb, lz_eps);
    std::vector<double> HW(W.size(), 0.0);
    sbd::mult(hii, W, HW, adet, bdet, bit_length, (size_t)L, 1, 1, helper, I0, I1, I2, h_comm, b_comm, t_comm);
    double E = 0.0, nrm = 0.0;
    sbd::InnerProduct(W, HW, E, b_comm);
    sbd::InnerProduct(W, W, nrm, b_comm);
    out.scalar("lanczos_energy", E / nrm);
  }

  if (want_dav) {
    std::vector<double> W;
    sbd::BasisInitVector(W, adet, bdet, 1, 1, h_comm, b_comm, t_comm, 0, 1729);
    auto td0 = std::chrono::steady_clock::now();
    sbd::Davidson(hii, W, adet, bdet, bit_length, (size_t)L, 1, 1, helper, I0, I1, I2, h_comm, b_comm, t_comm,
                  max_it, max_nb, eps, 86400.0);
    auto td1 = std::chrono::steady_clock::now();
    std::vector<double> HW(W.size(), 0.0);
    sbd::mult(hii, W, HW, adet, bdet, bit_length, (size_t)L, 1, 1, helper, I0, I1, I2, h_comm, b_comm, t_comm);
    double E = 0.0;
    sbd::InnerProduct(W, HW, E, b_comm);
    std::cout.precision(16);
    std::cout << " Energy = " << E << std::endl;
    out.scalar("t_davidson", std::chrono::duration<double>(td1 - td0).count());
    out.scalar("energy", E);
    out.f64("W", W);
    if (!savename.empty()) sbd::SaveWavefunction(savename, adet, bdet, 1, 1, h_comm, b_comm, t_comm, W);
    if (co_type != 0) {
      sbd::det_vector<size_t, sbd::det_kind::half> co_adet, co_bdet;
      if (co_type == 1 || co_type == 2) {
        if (co_ratio == 0.0) {
          sbd::CarryOverAdet(W, adet, bdet, 1, 1, b_comm, co_adet, co_threshold);
          sbd::CarryOverBdet(W, adet, bdet, 1, 1, b_comm, co_bdet, co_threshold);
        } else {
          double tw = 0.0;
          sbd::CarryOverAdet(W, adet, bdet, 1, 1, b_comm, static_cast<size_t>(co_ratio * adet.size()), co_adet, tw);
          out.scalar("truncated_a", tw);
          sbd::CarryOverBdet(W, adet, bdet, 1, 1, b_comm, static_cast<size_t>(co_ratio * bdet.size()), co_bdet, tw);
          out.scalar("truncated_b", tw);
        }
        if (co_type == 2) {
          sbd::det_vector<size_t, sbd::det_kind::half> ra, rb;
          sbd::SinglesExtendHalfdets(co_adet, co_bdet, bit_length, (size_t)L, 1, 1, b_comm, ra, rb);
          co_adet = ra;
          co_bdet = rb;
        }
      } else if (co_type == 3) {
        double total = 0.0;
        sbd::SinglesExtendHalfdets(W, adet, bdet, bit_length, (size_t)L, 1, 1, b_comm, co_threshold, co_adet, co_bdet,
                                   total);
        out.scalar("total_weight", total);
      }
      std::vector<size_t> a(co_adet.size() * co_adet.elem_size()), b(co_bdet.size() * co_bdet.elem_size());
      for (size_t i = 0; i < co_adet.size(); ++i)
        for (size_t w = 0; w < co_adet.elem_size(); ++w) a[i * co_adet.elem_size() + w] = co_adet[i][w];
      for (size_t i = 0; i < co_bdet.size(); ++i)
        for (size_t w = 0; w < co_bdet.elem_size(); ++w) b[i * co_bdet.elem_size() + w] = co_bdet[i][w];
      out.u64("co_adet_words", a);
      out.u64("co_bdet_words", b);
    }
  }

  if (!loadname.empty()) {
    std::vector<double> W;
    sbd::LoadWavefunction(loadname, adet, bdet, 1, 1, h_comm, b_comm, t_comm, W);
    out.f64("loaded_W", W);
  }
  MPI_Finalize();
  return 0;
}
