// sbdgb::tpb::diag with the reference's full argument list (sbdiag.h:151-163):
// wavefunction load/save, density, RDMs and carry-over strings.
//   tpb_diag_full --fcidump F --adetfile A [--bdetfile B] [--loadname X] [--savename Y] <diag flags>
// Prints the energy, the density sums, the carry-over strings and the traces
// of the RDM blocks.
#include <iostream>
#include <string>

#include "sbdgb/tpb.hpp"

int main(int argc, char **argv) {
  std::string fcidumpfile, adetfile, bdetfile, loadname, savename;
  for (int i = 1; i + 1 < argc; ++i) {
    std::string a(argv[i]);
    if (a == "--fcidump") fcidumpfile = argv[i + 1];
    if (a == "--adetfile") adetfile = argv[i + 1];
    if (a == "--bdetfile") bdetfile = argv[i + 1];
    if (a == "--loadname") loadname = argv[i + 1];
    if (a == "--savename") savename = argv[i + 1];
  }
  auto sbd_data = sbdgb::tpb::generate_sbd_data(argc, argv);
  sbdgb::FCIDump fcidump = sbdgb::LoadFCIDump(fcidumpfile);
  int L = 0;
  for (const auto &kv : fcidump.header)
    if (kv.first == "NORB") L = std::atoi(kv.second.c_str());
  auto adet = sbdgb::LoadAlphaDets(adetfile, L);
  auto bdet = bdetfile.empty() ? adet : sbdgb::LoadAlphaDets(bdetfile, L);
  double energy = 0.0;
  std::vector<double> density;
  std::vector<uint64_t> co_a, co_b;
  std::vector<std::vector<double>> one, two;
  sbdgb::tpb::diag(1, sbd_data, fcidump, adet, bdet, loadname, savename, energy, density, co_a, co_b, one, two);
  std::cout.precision(16);
  std::cout << " Energy = " << energy << std::endl;
  double na = 0.0, nb = 0.0;
  for (int io = 0; io < L; ++io) {
    na += density[2 * io];
    nb += density[2 * io + 1];
  }
  std::cout << " Density sums = " << na << " " << nb << std::endl;
  std::cout << " CarryOver alpha =";
  for (uint64_t v : co_a) std::cout << " " << v;
  std::cout << std::endl << " CarryOver beta =";
  for (uint64_t v : co_b) std::cout << " " << v;
  std::cout << std::endl;
  if (!one.empty()) {
    double t0 = 0.0, t1 = 0.0;
    for (int i = 0; i < L; ++i) {
      t0 += one[0][i + (size_t)L * i];
      t1 += one[1][i + (size_t)L * i];
    }
    std::cout << " RDM1 traces = " << t0 << " " << t1 << std::endl;
  }
  return 0;
}
