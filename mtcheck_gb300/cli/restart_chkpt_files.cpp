// restart_chkpt_files -- restart one checkpoint of a series from its files.
//
// The restart driver of the reference (src/restart_chkpt_files.cpp:19-201)
// on the GB300 library:
//   restart_chkpt_files restart_id num_chkpts num_tests chunk_size <mode> file_0 ... file_{n-1}
// The original file `file_<restart_id>` gives the buffer length; the chain is
// read from file_i + the approach's suffix (.full_chkpt, .basic.incr_chkpt,
// .hashlist.incr_chkpt, .hashtree.incr_chkpt), restarted `num_tests` times
// into device memory, and each time the buffer's digest is printed the way
// the reference does (calculate_digest_host, include/hash_functions.hpp:65-82)
// and the restart timing log <basename>.chunk_size.<c>.restart_timing.csv is
// appended (src/tree_approach.cpp:1787-1808).  Every tree flag runs the tree
// deduplicator, as in the reference driver.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "mtcheck/deduplicator.hpp"

namespace {

int get_mode(int argc, char** argv) {  // src/utils.cpp:15-36
  static const struct {
    const char* flag;
    int mode;
  } flags[] = {{"--run-full-chkpt", MTC_FULL},
               {"--run-basic-chkpt", MTC_BASIC},
               {"--run-list-chkpt", MTC_LIST},
               {"--run-tree-chkpt", MTC_TREE},
               {"--run-tree-low-offset-ref-chkpt", MTC_TREE_LOW_OFFSET_REF},
               {"--run-tree-low-offset-chkpt", MTC_TREE_LOW_OFFSET},
               {"--run-tree-low-root-ref-chkpt", 7},
               {"--run-tree-low-root-chkpt", 8}};
  for (int i = 0; i < argc; i++)
    for (const auto& f : flags)
      if (std::strcmp(argv[i], f.flag) == 0) return f.mode;
  return 0;
}

std::string basename_of(const std::string& path) {
  const size_t p = path.rfind('/');
  return p == std::string::npos ? path : path.substr(p + 1);
}

std::vector<uint8_t> read_file(const std::string& path) {
  std::ifstream f(path, std::ios::in | std::ios::binary | std::ios::ate);
  if (!f) throw mtcheck::Error(MTC_EINVAL, "cannot open " + path);
  const std::streamsize n = f.tellg();
  f.seekg(0);
  std::vector<uint8_t> v((size_t)n);
  if (n && !f.read(reinterpret_cast<char*>(v.data()), n)) throw mtcheck::Error(MTC_EINVAL, "cannot read " + path);
  return v;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s restart_id num_chkpts num_tests chunk_size <mode> chkpt_files...\n", argv[0]);
    return 2;
  }
  const uint32_t restart_id = static_cast<uint32_t>(std::atoi(argv[1]));
  const uint32_t num_chkpts = static_cast<uint32_t>(std::atoi(argv[2]));
  const uint32_t num_tests = static_cast<uint32_t>(std::atoi(argv[3]));
  const uint32_t chunk_size = static_cast<uint32_t>(std::atoi(argv[4]));
  const int mode = get_mode(argc, argv);
  if (mode == 0) {
    std::printf("ERROR: Incorrect mode\n");
    return 2;
  }
  const uint32_t arg_offset = 1;  // the mode flag sits at argv[5]
  if ((uint32_t)argc < 5 + arg_offset + num_chkpts || restart_id >= num_chkpts) {
    std::fprintf(stderr, "expected %u checkpoint files and restart_id < num_chkpts\n", num_chkpts);
    return 2;
  }
  std::vector<std::string> files;
  for (uint32_t i = 0; i < num_chkpts; i++) files.push_back(argv[5 + arg_offset + i]);
  try {
    const char* suffix = ".hashtree.incr_chkpt";
    const char* label = "Hashtree digest:       ";
    std::unique_ptr<mtcheck::BaseDeduplicator> dedup;
    if (mode == MTC_FULL) {
      dedup.reset(new mtcheck::FullDeduplicator(chunk_size));
      suffix = ".full_chkpt";
      label = "Full chkpt digest:     ";
    } else if (mode == MTC_BASIC) {
      dedup.reset(new mtcheck::BasicDeduplicator(chunk_size));
      suffix = ".basic.incr_chkpt";
      label = "Basic Hashlist digest: ";
    } else if (mode == MTC_LIST) {
      dedup.reset(new mtcheck::ListDeduplicator(chunk_size));
      suffix = ".hashlist.incr_chkpt";
      label = "Hashlist digest:       ";
    } else {
      dedup.reset(new mtcheck::TreeDeduplicator(chunk_size));
    }
    // the restarted buffer has the length of the original checkpoint file
    size_t filesize = 0;
    {
      std::ifstream f(files[restart_id], std::ios::in | std::ios::binary | std::ios::ate);
      if (!f) throw mtcheck::Error(MTC_EINVAL, "cannot open " + files[restart_id]);
      filesize = static_cast<size_t>(f.tellg());
    }
    uint8_t* reference = nullptr;
    if (cudaMalloc(&reference, filesize ? filesize : 1) != cudaSuccess)
      throw mtcheck::Error(MTC_ENOMEM, "cannot allocate the device buffer");
    std::vector<uint8_t> host(filesize);
    std::string logname = basename_of(files[restart_id]);
    for (uint32_t t = 0; t < num_tests; t++) {
      cudaMemset(reference, 0, filesize);
      std::vector<std::vector<uint8_t>> chkpts;
      for (uint32_t i = 0; i < num_chkpts; i++) chkpts.push_back(read_file(files[i] + suffix));
      dedup->restart(reference, filesize, chkpts, logname, restart_id);
      if (cudaMemcpy(host.data(), reference, filesize, cudaMemcpyDeviceToHost) != cudaSuccess)
        throw mtcheck::Error(MTC_ECUDA, "device to host copy failed");
      uint8_t d[16];
      char hex[37];
      mtcheck::check(mtc_digest_host(MTC_HASH_MURMUR3, host.data(), filesize, d));
      mtcheck::check(mtc_digest_hex(d, hex));
      std::cout << label << hex << std::endl;
    }
    cudaFree(reference);
  } catch (const mtcheck::Error& e) {
    std::fprintf(stderr, "restart_chkpt_files: %s\n", e.what());
    return 1;
  }
  return 0;
}
