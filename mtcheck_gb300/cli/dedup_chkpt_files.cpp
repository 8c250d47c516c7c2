// dedup_chkpt_files -- deduplicate a series of checkpoint files.
//
// The command-line driver of the reference (src/dedup_files.cpp:9-108) on the
// GB300 library:
//   dedup_chkpt_files chunk_size num_chkpts <mode> file_0 ... file_{n-1}
// mode: --run-full-chkpt | --run-basic-chkpt | --run-list-chkpt |
//       --run-tree-chkpt and the other tree flags of get_mode()
//       (src/utils.cpp:3-36); like the reference driver, every tree flag runs
//       the tree deduplicator (src/dedup_files.cpp:68-70, :100-104).
// Each file is loaded into device memory and checkpointed in order, the first
// as the baseline.  The incremental checkpoint of <file> is written to
// <file>.full_chkpt / .basic.incr_chkpt / .hashlist.incr_chkpt /
// .hashtree.incr_chkpt, and the CSV logs of the reference to
// <basename(file)>.chunk_size.<c>{.csv,.size.csv,.timing.csv} in the working
// directory (src/dedup_files.cpp:84-99).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "mtcheck/deduplicator.hpp"

namespace {

void print_mode_help() {  // src/utils.cpp:3-13
  std::printf("Modes: \n");
  std::printf("Full checkpoint:                                   --run-full-chkpt\n");
  std::printf("Basic checkpoint:                                  --run-basic-chkpt\n");
  std::printf("List checkpoint:                                   --run-list-chkpt\n");
  std::printf("Tree checkpoint:                                   --run-tree-chkpt\n");
  std::printf("Tree checkpoint lowest offset reference algorithm: --run-tree-low-offset-ref-chkpt\n");
  std::printf("Tree checkpoint lowest offset algorithm:           --run-tree-low-offset-chkpt\n");
  std::printf("Tree checkpoint lowest root reference algorithm:   --run-tree-low-root-ref-chkpt\n");
  std::printf("Tree checkpoint lowest root algorithm:             --run-tree-low-root-chkpt\n");
}

// get_mode (src/utils.cpp:15-36): 0 when no flag matches
int get_mode(int argc, char** argv) {
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

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s chunk_size num_chkpts <mode> chkpt_files...\n", argv[0]);
    print_mode_help();
    return 2;
  }
  const uint32_t chunk_size = static_cast<uint32_t>(std::atoi(argv[1]));
  const uint32_t num_chkpts = static_cast<uint32_t>(std::atoi(argv[2]));
  const int mode = get_mode(argc, argv);
  if (mode == 0) {
    std::printf("ERROR: Incorrect mode\n");
    print_mode_help();
    return 2;
  }
  const uint32_t arg_offset = 1;  // the mode flag sits at argv[3]
  if ((uint32_t)argc < 3 + arg_offset + num_chkpts) {
    std::fprintf(stderr, "expected %u checkpoint files\n", num_chkpts);
    return 2;
  }
  try {
    std::unique_ptr<mtcheck::BaseDeduplicator> dedup;
    const char* suffix = ".hashtree.incr_chkpt";
    if (mode == MTC_FULL) {
      dedup.reset(new mtcheck::FullDeduplicator(chunk_size));
      suffix = ".full_chkpt";
    } else if (mode == MTC_BASIC) {
      dedup.reset(new mtcheck::BasicDeduplicator(chunk_size));
      suffix = ".basic.incr_chkpt";
    } else if (mode == MTC_LIST) {
      dedup.reset(new mtcheck::ListDeduplicator(chunk_size));
      suffix = ".hashlist.incr_chkpt";
    } else {
      dedup.reset(new mtcheck::TreeDeduplicator(chunk_size));
    }
    uint8_t* current = nullptr;
    size_t capacity = 0;
    std::vector<char> host;
    for (uint32_t idx = 0; idx < num_chkpts; idx++) {
      const std::string path = argv[3 + arg_offset + idx];
      std::ifstream f(path, std::ios::in | std::ios::binary | std::ios::ate);
      if (!f) throw mtcheck::Error(MTC_EINVAL, "cannot open " + path);
      const size_t data_len = static_cast<size_t>(f.tellg());
      f.seekg(0);
      host.resize(data_len);
      if (data_len && !f.read(host.data(), (std::streamsize)data_len))
        throw mtcheck::Error(MTC_EINVAL, "cannot read " + path);
      if (data_len > capacity) {
        if (current) cudaFree(current);
        if (cudaMalloc(&current, data_len ? data_len : 1) != cudaSuccess)
          throw mtcheck::Error(MTC_ENOMEM, "cannot allocate the device buffer");
        capacity = data_len;
      }
      if (cudaMemcpy(current, host.data(), data_len, cudaMemcpyHostToDevice) != cudaSuccess)
        throw mtcheck::Error(MTC_ECUDA, "host to device copy failed");
      std::string filename = path + suffix;
      std::string logname = basename_of(path);
      dedup->checkpoint(current, data_len, filename, logname, idx == 0);
    }
    if (current) cudaFree(current);
  } catch (const mtcheck::Error& e) {
    std::fprintf(stderr, "dedup_chkpt_files: %s\n", e.what());
    return 1;
  }
  return 0;
}
