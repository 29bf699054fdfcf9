// Several problems (FCIDUMP + alpha/beta string files each) solved together
// through the C++ mirror's BatchDavidson, in FP64 and in the mixed form.
//   batch_solve F1 A1 B1 [F2 A2 B2 ...]
// prints "problem i fp64 E mixed E" per problem (ground energies).
#include <cstdio>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "sbdgb/tpb.hpp"

int main(int argc, char **argv) {
  if (argc < 4 || (argc - 1) % 3 != 0) {
    std::cerr << "usage: batch_solve FCIDUMP ADETS BDETS [...]" << std::endl;
    return 2;
  }
  sbdgb::Context ctx(0);
  std::vector<std::unique_ptr<sbdgb::Problem>> owned;
  std::vector<sbdgb::Problem *> problems;
  for (int i = 1; i + 2 < argc; i += 3) {
    sbdgb::FCIDump fcidump = sbdgb::LoadFCIDump(argv[i]);
    int L = 0;
    for (const auto &kv : fcidump.header)
      if (kv.first == "NORB") L = std::atoi(kv.second.c_str());
    auto adet = sbdgb::LoadAlphaDets(argv[i + 1], L);
    auto bdet = sbdgb::LoadAlphaDets(argv[i + 2], L);
    owned.emplace_back(new sbdgb::Problem(ctx, sbdgb::SetupIntegrals(fcidump), adet, bdet));
    problems.push_back(owned.back().get());
  }
  auto e64 = sbdgb::BatchDavidson(problems, 1, 16, 1e-10);
  auto emx = sbdgb::BatchDavidson(problems, 1, 16, 1e-10, 100, SBDGB_MIXED);
  std::cout.precision(16);
  for (size_t i = 0; i < problems.size(); ++i)
    std::cout << "problem " << i << " fp64 " << e64[i][0] << " mixed " << emx[i][0] << std::endl;
  return 0;
}
