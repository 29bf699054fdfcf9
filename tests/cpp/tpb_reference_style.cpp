// A caller written the way the reference's own TPB users are, against
// namespace sbd, compiled against the GB300 engine's reference-shaped header:
// the only change from a reference build is the namespace alias below.
//
//   tpb_reference_style --mode diag|diagfile|inner --fcidump F --adetfile A
//                       [--bdetfile B] [--block NB --iteration IT --tolerance EPS]
//
//   diag      LoadFCIDump + MpiBcast, LoadAlphaDets + sort_bitarray + MpiBcast,
//             tpb::diag(comm, sbd_data, fcidump, adet, bdet, loadname, savename,
//             energy, density, co_adet, co_bdet, one_p_rdm, two_p_rdm)
//   diagfile  tpb::diag(comm, sbd_data, fcidumpfile, adetfile, ...)
//   inner     MakeHelpers, SetupIntegrals, makeQChamDiagTerms, Davidson and mult
//             with their 10-19 argument lists, and the MultBase operator
#include <cmath>
#include <iostream>
#include <string>
#include <vector>

#include "mpi.h"
#include "sbdgb/sbd_compat.hpp"

namespace sbd = sbdgb;

int main(int argc, char *argv[]) {
  int provided;
  MPI_Init_thread(&argc, &argv, MPI_THREAD_FUNNELED, &provided);
  MPI_Comm comm = MPI_COMM_WORLD;
  int mpi_rank;
  MPI_Comm_rank(comm, &mpi_rank);

  auto sbd_data = sbd::tpb::generate_sbd_data(argc, argv);
  std::string mode("diag"), adetfile("alphadets.txt"), bdetfile, fcidumpfile("fcidump.txt"), loadname, savename;
  for (int i = 0; i < argc; i++) {
    if (std::string(argv[i]) == "--mode") mode = std::string(argv[++i]);
    else if (std::string(argv[i]) == "--adetfile") adetfile = std::string(argv[++i]);
    else if (std::string(argv[i]) == "--bdetfile") bdetfile = std::string(argv[++i]);
    else if (std::string(argv[i]) == "--fcidump") fcidumpfile = std::string(argv[++i]);
    else if (std::string(argv[i]) == "--loadname") loadname = std::string(argv[++i]);
    else if (std::string(argv[i]) == "--savename") savename = std::string(argv[++i]);
  }

  int L = 0, N = 0;
  double energy = 0.0;
  std::vector<double> density;
  sbd::det_vector<size_t, sbd::det_kind::half> co_adet, co_bdet;
  std::vector<std::vector<double>> one_p_rdm, two_p_rdm;
  std::cout.precision(16);

  if (mode == "diagfile") {
    sbd::tpb::diag(comm, sbd_data, fcidumpfile, adetfile, loadname, savename, energy, density, co_adet, co_bdet,
                   one_p_rdm, two_p_rdm);
    std::cout << " Sample-based diagonalization: Energy = " << energy << std::endl;
    MPI_Finalize();
    return 0;
  }

  sbd::FCIDump fcidump;
  if (mpi_rank == 0) fcidump = sbd::LoadFCIDump(fcidumpfile);
  sbd::MpiBcast(fcidump, 0, comm);
  for (const auto &[key, value] : fcidump.header) {
    if (key == std::string("NORB")) L = std::atoi(value.c_str());
    if (key == std::string("NELEC")) N = std::atoi(value.c_str());
  }
  sbd::det_vector<size_t, sbd::det_kind::half> adet, bdet;
  if (mpi_rank == 0) {
    sbd::LoadAlphaDets(adetfile, adet, sbd_data.bit_length, L);
    sbd::sort_bitarray(adet);
  }
  sbd::MpiBcast(adet, 0, comm);
  if (bdetfile.empty()) {
    bdet = adet;
  } else {
    if (mpi_rank == 0) {
      sbd::LoadAlphaDets(bdetfile, bdet, sbd_data.bit_length, L);
      sbd::sort_bitarray(bdet);
    }
    sbd::MpiBcast(bdet, 0, comm);
  }

  if (mode == "diag") {
    sbd::tpb::diag(comm, sbd_data, fcidump, adet, bdet, loadname, savename, energy, density, co_adet, co_bdet,
                   one_p_rdm, two_p_rdm);
    std::cout << " Sample-based diagonalization: Energy = " << energy << std::endl;
    double occ = 0.0;
    for (size_t i = 0; i < density.size(); i++) occ += density[i];
    std::cout << " Sample-based diagonalization: electrons = " << occ << std::endl;
    std::cout << " Sample-based diagonalization: carryover bitstrings = [";
    for (size_t i = 0; i < std::min(co_adet.size(), static_cast<size_t>(4)); i++)
      std::cout << ((i == 0) ? "" : ", ") << sbd::makestring(co_adet[i], sbd_data.bit_length, L);
    std::cout << "], size = " << co_adet.size() << std::endl;
    MPI_Finalize();
    return 0;
  }

  // mode inner: the operator-level entry points
  std::vector<sbd::TaskHelpers> helper;
  sbd::MakeHelpers(adet, bdet, sbd_data.bit_length, L, helper, comm, comm, comm, 1, 1);
  double I0;
  sbd::oneInt<double> I1;
  sbd::twoInt<double> I2;
  sbd::SetupIntegrals(fcidump, L, N, I0, I1, I2);
  std::vector<double> hii;
  sbd::makeQChamDiagTerms(adet, bdet, sbd_data.bit_length, L, helper, I0, I1, I2, hii, comm, comm, comm);
  std::vector<double> W(adet.size() * bdet.size(), 0.0);
  W[0] = 1.0;  // the first determinant, as the reference's init 0
  sbd::Davidson(hii, W, adet, bdet, sbd_data.bit_length, L, 1, 1, helper, I0, I1, I2, comm, comm, comm,
                sbd_data.max_it, sbd_data.max_nb, sbd_data.eps, sbd_data.max_time);
  std::vector<double> HW(W.size(), 0.0);
  sbd::mult(hii, W, HW, adet, bdet, sbd_data.bit_length, L, 1, 1, helper, I0, I1, I2, comm, comm, comm);
  double e = 0.0, n2 = 0.0;
  for (size_t i = 0; i < W.size(); i++) {
    e += W[i] * HW[i];
    n2 += W[i] * W[i];
  }
  std::cout << " Davidson energy = " << e / n2 << std::endl;
  // the same product through the operator interface
  sbd::MultTPB<double> op(adet, bdet, sbd_data.bit_length, L, helper, I0, I1, I2, comm, comm, comm);
  sbd::MultBase<double> &base = op;
  std::vector<double> HW2(W.size(), 0.0);
  base.run(hii, W, HW2);
  double dmax = 0.0, hmax = 0.0;
  for (size_t i = 0; i < W.size(); i++) {
    dmax = std::max(dmax, std::fabs(HW2[i] - HW[i]));
    hmax = std::max(hmax, std::fabs(HW[i]));
  }
  std::cout << " MultBase relative difference = " << dmax / hmax << std::endl;
  std::cout << " helper singles = " << helper[0].SinglesFromAlpha_flat.size() << std::endl;
  MPI_Finalize();
  return 0;
}
