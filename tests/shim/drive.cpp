// Calls the INTEGRATION.md shim the way SCESS's call sites do
// (SolveRCCSD_DIIS, then RCCSD_TriplesCorrection on its amplitudes).
// Usage: drive <eri.bin> <eps.bin> <nmo> <nocc>; the .bin files hold the
// column-major nmo^4 eri and the nmo orbital energies as raw doubles.
// Prints "converged E_CCSD E_T" and the console lines to stderr.
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "Quantum/CC/CC.h"

using namespace SCESS::CC;

static bool read_doubles(const char *path, double *dst, size_t n) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  const size_t got = std::fread(dst, sizeof(double), n, f);
  std::fclose(f);
  return got == n;
}

int main(int argc, char **argv) {
  if (argc != 5) return 2;
  const Eigen::Index n = std::atol(argv[3]), o = std::atol(argv[4]);
  TEITensor eri(n, n, n, n);
  Eigen::VectorXd eps(n);
  if (!read_doubles(argv[1], eri.data(), (size_t)(n * n * n * n)) ||
      !read_doubles(argv[2], eps.data(), (size_t)n))
    return 3;
  std::stringstream console;
  DH::Thread thread;
  try {
    const RCCSD_Wfn w = SolveRCCSD_DIIS(eri, eps, o, nullptr, &thread, &console);
    const double et = w.converged ? RCCSD_TriplesCorrection(eri, eps, o, w.t1, w.t2, &thread) : 0.0;
    std::cerr << console.str();
    std::printf("%d %.15f %.15f\n", w.converged ? 1 : 0, w.E_CCSD, et);
  } catch (const std::exception &e) {
    std::cerr << "error: " << e.what() << "\n";
    return 4;
  }
  return 0;
}
