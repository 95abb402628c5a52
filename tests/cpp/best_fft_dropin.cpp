// Caller-side check of the C++ drop-in: the reference's call shape
// (test/main.cpp:57, best_fft<FieldT>(v, omg)) on the new element types.
// Usage: best_fft_dropin <field 0|1|2> <log_n> <in.bin> <omega.bin> <out.bin>
// Reads n elements and omega (raw little-endian limbs), runs best_fft in
// place, then the inverse round trip through gsn::transform, and writes the
// forward result.  Exit 0 on success, 2 if the round trip fails, 1 on error.
#include <cstdio>
#include <cstring>
#include <vector>

#include "gsn_best_fft.h"

template <class F>
static int run(int log_n, const char* in, const char* om, const char* out) {
  const size_t n = size_t(1) << log_n;
  std::vector<F> v(n), orig(n);
  F omg;
  FILE* fi = std::fopen(in, "rb");
  FILE* fo = std::fopen(om, "rb");
  if (!fi || !fo) return 1;
  if (std::fread(v.data(), sizeof(F), n, fi) != n || std::fread(&omg, sizeof(F), 1, fo) != 1) return 1;
  std::fclose(fi);
  std::fclose(fo);
  orig = v;
  best_fft<F>(v, omg);  // the reference's entry point
  std::vector<F> w = v;
  gsn::transform(w, &omg, GSN_INVERSE);
  if (std::memcmp(w.data(), orig.data(), n * sizeof(F)) != 0) return 2;
  // several vectors at once through the pipelined host path: each equals the single call
  std::vector<F> m0 = orig, m1 = orig, m2 = orig;
  gsn::best_fft_many<F>({&m0, &m1, &m2}, omg);
  for (const std::vector<F>* m : {&m0, &m1, &m2})
    if (std::memcmp(m->data(), v.data(), n * sizeof(F)) != 0) return 2;
  FILE* fw = std::fopen(out, "wb");
  if (!fw) return 1;
  std::fwrite(v.data(), sizeof(F), n, fw);
  std::fclose(fw);
  // errors are reported, not fatal: a wrong root throws gsn::Error
  try {
    F bad{};
    bad.im_rep[0] = 2;
    best_fft<F>(v, bad);
    return 1;
  } catch (const gsn::Error& e) {
    if (e.code != GSN_ERR_OMEGA) return 1;
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 6) return 1;
  const int field = std::atoi(argv[1]);
  const int log_n = std::atoi(argv[2]);
  try {
    switch (field) {
      case 0: return run<gsn::Fp32>(log_n, argv[3], argv[4], argv[5]);
      case 1: return run<gsn::FrBLS12_381>(log_n, argv[3], argv[4], argv[5]);
      case 2: return run<gsn::FrMNT4_753>(log_n, argv[3], argv[4], argv[5]);
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
  }
  return 1;
}
