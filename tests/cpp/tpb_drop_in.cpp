// Drop-in use of the C++ mirror: the same call sequence as the reference's TPB
// app (apps/chemistry_tpb_selected_basis_diagonalization/main.cc:127-191):
// load FCIDUMP, load and sort the alpha/beta string files, run diag.
//   tpb_drop_in --fcidump F --adetfile A [--bdetfile B] [--method 0|2] --block NB --iteration IT
//               --tolerance EPS
#include <cstdio>
#include <iostream>
#include <string>

#include "sbdgb/tpb.hpp"

int main(int argc, char **argv) {
  std::string fcidumpfile = "fcidump.txt", adetfile = "alphadets.txt", bdetfile;
  for (int i = 1; i + 1 < argc; ++i) {
    std::string a(argv[i]);
    if (a == "--fcidump") fcidumpfile = argv[i + 1];
    if (a == "--adetfile") adetfile = argv[i + 1];
    if (a == "--bdetfile") bdetfile = argv[i + 1];
  }
  auto sbd_data = sbdgb::tpb::generate_sbd_data(argc, argv);
  sbdgb::FCIDump fcidump = sbdgb::LoadFCIDump(fcidumpfile);
  int L = 0;
  for (const auto &kv : fcidump.header)
    if (kv.first == "NORB") L = std::atoi(kv.second.c_str());
  auto adet = sbdgb::LoadAlphaDets(adetfile, L);
  auto bdet = bdetfile.empty() ? adet : sbdgb::LoadAlphaDets(bdetfile, L);
  double energy = 0.0;
  std::vector<double> W, density;
  sbdgb::tpb::diag(1, sbd_data, fcidump, adet, bdet, energy, &W, nullptr, &density);
  // <W|H|W> through the mult entry point, as the reference reports it (sbdiag.h:488-526)
  sbdgb::Context ctx(sbd_data.device);
  sbdgb::Problem p(ctx, sbdgb::SetupIntegrals(fcidump), adet, bdet);
  std::vector<double> hii, HW(W.size(), 0.0);
  sbdgb::makeQChamDiagTerms(p, hii);
  sbdgb::mult(hii, W, HW, p);
  double e = 0.0;
  for (size_t i = 0; i < W.size(); ++i) e += W[i] * HW[i];
  std::cout.precision(16);
  std::cout << " Energy = " << e << std::endl;
  std::cout << " Solver energy = " << energy << std::endl;
  double na = 0.0, nb = 0.0;
  for (int io = 0; io < L; ++io) {
    na += density[2 * io];
    nb += density[2 * io + 1];
  }
  std::cout << " Density sums = " << na << " " << nb << std::endl;
  return 0;
}
