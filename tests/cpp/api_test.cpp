// Exercises include/mtcheck/deduplicator.hpp the way the reference's own tests
// exercise BaseDeduplicator: test/test_case_XX.cpp (two 8-byte checkpoints with
// 1-byte chunks, region counts and restart digests) and test/tree_chkpt.cpp
// (a chain of random buffers, each restarted and compared by digest).
// Input on stdin, one known-answer case per line: "<chunk> <step0> <step1> <fo> <shift>".
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "mtcheck/deduplicator.hpp"

static std::string digest_str(const std::vector<uint8_t>& h) {
  uint8_t d[16];
  char out[37];
  mtc_digest_host(MTC_HASH_MURMUR3, h.data(), h.size(), d);
  mtc_digest_hex(d, out);
  return out;
}

static std::vector<uint8_t> to_host(const uint8_t* dev, size_t n) {
  std::vector<uint8_t> h(n);
  cudaMemcpy(h.data(), dev, n, cudaMemcpyDeviceToHost);
  return h;
}

static int known_answer(uint32_t chunk, const std::string& s0, const std::string& s1, size_t fo, size_t sh) {
  uint8_t *d0, *d1, *out;
  cudaMalloc(&d0, 8);
  cudaMalloc(&d1, 8);
  cudaMalloc(&out, 8);
  cudaMemcpy(d0, s0.data(), 8, cudaMemcpyHostToDevice);
  cudaMemcpy(d1, s1.data(), 8, cudaMemcpyHostToDevice);
  mtcheck::TreeDeduplicator deduplicator(chunk);
  std::vector<std::vector<uint8_t>> incr_chkpts;
  std::vector<uint8_t> diff_h;
  std::string null("/dev/null/");
  int res = 0;
  deduplicator.checkpoint(d0, 8, diff_h, true);
  incr_chkpts.push_back(diff_h);
  deduplicator.restart(out, 8, incr_chkpts, null, 0);
  if (digest_str(to_host(out, 8)) != digest_str(std::vector<uint8_t>(s0.begin(), s0.end()))) res = 1;
  deduplicator.checkpoint(d1, 8, diff_h, false);
  incr_chkpts.push_back(diff_h);
  deduplicator.restart(out, 8, incr_chkpts, null, 1);
  if (digest_str(to_host(out, 8)) != digest_str(std::vector<uint8_t>(s1.begin(), s1.end()))) res = 2;
  if (deduplicator.num_first_ocur() != fo || deduplicator.num_shift_dupl() != sh) res = 3;
  std::printf("case %s %s -> (%zu, %zu) expected (%zu, %zu): %s\n", s0.c_str(), s1.c_str(),
              deduplicator.num_first_ocur(), deduplicator.num_shift_dupl(), fo, sh, res ? "FAIL" : "ok");
  cudaFree(d0);
  cudaFree(d1);
  cudaFree(out);
  return res;
}

template <class D>
static int chain(const char* name, uint32_t chunk, uint32_t nchkpts) {
  const size_t len = 1 << 20;
  std::mt19937 rng(1931);
  std::vector<uint8_t> h(len);
  uint8_t *data, *out;
  cudaMalloc(&data, len);
  cudaMalloc(&out, len);
  D deduplicator(chunk);
  std::vector<std::vector<uint8_t>> incr_chkpts;
  std::string null("/dev/null/");
  int res = 0;
  for (uint32_t i = 0; i < nchkpts; i++) {
    for (auto& b : h) b = (uint8_t)(rng() & 0xff);
    cudaMemcpy(data, h.data(), len, cudaMemcpyHostToDevice);
    std::string correct = digest_str(h);
    std::vector<uint8_t> diff_h;
    deduplicator.checkpoint(data, len, diff_h, i == 0);
    incr_chkpts.push_back(diff_h);
    cudaMemset(out, 0, len);
    deduplicator.restart(out, len, incr_chkpts, null, i);
    if (digest_str(to_host(out, len)) != correct) res = 1;
  }
  std::printf("%s chain of %u checkpoints: %s\n", name, nchkpts, res ? "FAIL" : "ok");
  cudaFree(data);
  cudaFree(out);
  return res;
}

int main() {
  int fails = 0;
  std::string line;
  while (std::getline(std::cin, line)) {
    std::istringstream in(line);
    uint32_t chunk;
    std::string s0, s1;
    size_t fo, sh;
    if (!(in >> chunk >> s0 >> s1 >> fo >> sh)) continue;
    fails += known_answer(chunk, s0, s1, fo, sh) != 0;
  }
  try {
    fails += chain<mtcheck::TreeDeduplicator>("tree", 128, 10);
    fails += chain<mtcheck::ListDeduplicator>("list", 128, 10);
    fails += chain<mtcheck::BasicDeduplicator>("basic", 128, 10);
    fails += chain<mtcheck::FullDeduplicator>("full", 128, 10);
    // errors surface as exceptions with the C ABI status
    mtcheck::TreeDeduplicator d(128);
    std::vector<std::vector<uint8_t>> empty(1);
    uint8_t* out;
    cudaMalloc(&out, 64);
    std::string null("/dev/null/");
    bool threw = false;
    try {
      d.restart(out, 64, empty, null, 0);
    } catch (const mtcheck::Error& e) {
      threw = e.code() == MTC_ECORRUPT;
    }
    cudaFree(out);
    std::printf("corrupt chain raises mtcheck::Error: %s\n", threw ? "ok" : "FAIL");
    fails += !threw;
  } catch (const std::exception& e) {
    std::printf("unexpected exception: %s\n", e.what());
    fails++;
  }
  std::printf("%d failures\n", fails);
  return fails ? 1 : 0;
}
