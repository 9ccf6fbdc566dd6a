// Host build of the packer's FASTA classifier (mczi_gb300/csrc/fasta_classify.cuh,
// the code the device kernels run) checked against its byte-by-byte rule on
// random 32-byte chunks: line state after the chunk, base count and break
// flags, the codes of every base in order, fragment starts, the carried break.
// Usage: pack_classify_fuzz <iterations>; exit status 0 when all agree.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "fasta_classify.cuh"

using namespace mczi::fasta;

int main(int argc, char** argv) {
  const long iters = argc > 1 ? std::atol(argv[1]) : 1000000;
  std::mt19937_64 rng(12345);
  static const char alpha[] = "ACGTacgtNn>\n\r-xACGTACGTACGT";
  long bad = 0;
  for (long it = 0; it < iters; it++) {
    alignas(16) uint8_t b[32];
    const int mode = (int)(it % 4);
    for (int i = 0; i < 32; i++) {
      if (mode == 0) b[i] = (uint8_t)alpha[rng() % (sizeof(alpha) - 1)];
      else if (mode == 1) b[i] = (rng() % 40 == 0) ? '\n' : (uint8_t)"ACGT"[rng() % 4];
      else if (mode == 2) b[i] = (uint8_t)(rng() & 0xff);
      else b[i] = (rng() % 10 == 0) ? (uint8_t)">\n\rN"[rng() % 4] : (uint8_t)"ACGTacgt"[rng() % 8];
    }
    const uint32_t st0 = (uint32_t)(rng() % 3);
    const uint32_t pend0 = (uint32_t)(rng() & 1);
    // the byte rule
    uint32_t st = st0, pend = pend0, nb = 0, fb = 0, lb = 0, starts = 0;
    uint32_t code[32];
    int n = 0;
    for (int i = 0; i < 32; i++) {
      const uint32_t x = step_fasta(b[i], st);
      if (x < 4) {
        nb++;
        lb = 0;
        if (pend) starts |= 1u << n;
        pend = 0;
        code[n++] = x;
      } else if (x == 4) {
        if (nb == 0) fb = 1;
        lb = 1;
        pend = 1;
      }
    }
    // the mask path
    uint32_t st2 = st0, pend2 = pend0, nb2, fb2, lb2, starts2 = 0;
    const Fasta32 f = fasta32(b, st2);
    fasta32_counts(f, &nb2, &fb2, &lb2);
    uint32_t code2[32];
    int n2 = 0;
    bool ok = true;
    fasta32_runs(f, pend2, [&](int len, uint64_t run, bool start) {
      if (n2 + len > 32) { ok = false; return; }
      if (start) starts2 |= 1u << n2;
      for (int t = 0; t < len; t++) code2[n2 + t] = (uint32_t)(run >> (62 - 2 * t)) & 3u;
      n2 += len;
    });
    ok = ok && st2 == st && nb2 == nb && n2 == n && pend2 == pend && starts2 == starts &&
         (nb == 0 ? lb2 == lb : (fb2 == fb && lb2 == lb));
    for (int t = 0; ok && t < n; t++) ok = code2[t] == code[t];
    if (!ok && ++bad <= 5) std::printf("mismatch at iteration %ld (state %u)\n", it, st0);
  }
  std::printf("%ld chunks, %ld mismatches\n", iters, bad);
  return bad ? 1 : 0;
}
