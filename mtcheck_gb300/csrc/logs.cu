// logs.cu -- CSV logs with the columns and formatting of the reference.
#include <cstring>
#include <fstream>

#include "logs.hpp"

namespace mtc {

static const char* approach_name(int mode) {
  switch (mode) {
    case MODE_FULL: return "Full";
    case MODE_BASIC: return "Basic";
    case MODE_LIST: return "List";
    default: return "Tree";
  }
}

// src/utils.cpp:38-124 (the values it writes; the STDOUT_PRINT lines are off
// by default in the reference)
static void write_metadata_breakdown(std::fstream& fs, const HeaderHost& h, const uint8_t* buf, uint64_t len,
                                     uint32_t num_chkpts) {
  fs << sizeof(HeaderHost) << "," << (size_t)h.num_first_ocur * sizeof(uint32_t) << ",";
  if (h.ref_id != h.chkpt_id) {
    fs << 2 * sizeof(uint32_t) * h.num_prior_chkpts;
    for (uint32_t i = 0; i < num_chkpts; i++) {
      if (i < h.num_prior_chkpts) {
        uint32_t num = 0;
        uint64_t off = sizeof(HeaderHost) + (uint64_t)h.num_first_ocur * 4 + (uint64_t)i * 8;
        if (off + 8 <= len) std::memcpy(&num, buf + off + 4, 4);
        fs << "," << (size_t)num * 2 * sizeof(uint32_t);
      } else {
        fs << "," << 0;
      }
    }
    fs << std::endl;
  } else {
    fs << 0 << ",";
    fs << (size_t)h.num_shift_dupl * 2 * sizeof(uint32_t);
    for (uint32_t i = 1; i < num_chkpts; i++) fs << "," << 0;
    fs << std::endl;
  }
}

void write_chkpt_log(const Engine& e, const HeaderHost& header, const uint8_t* diff, uint64_t diff_len,
                     const std::string& logname) {
  const std::string cs = std::to_string(e.chunk_size());
  std::fstream result_data, timing_file, size_file;
  result_data.open(logname + ".chunk_size." + cs + ".csv", std::fstream::ate | std::fstream::out | std::fstream::app);
  size_file.open(logname + ".chunk_size." + cs + ".size.csv", std::fstream::out | std::fstream::app);
  timing_file.open(logname + ".chunk_size." + cs + ".timing.csv", std::fstream::out | std::fstream::app);
  if (result_data.tellp() == 0) {
    result_data << "Approach,Chkpt ID,Chunk Size,Uncompressed Size,Compressed Size,Data Size,Metadata Size,Setup "
                   "Time,Comparison Time,Gather Time,Write Time"
                << std::endl;
  }
  const char* name = approach_name(e.mode());
  result_data << name << "," << e.current_id << "," << e.chunk_size() << "," << e.data_len << ","
              << e.datasizes[0] + e.datasizes[1] << "," << e.datasizes[0] << "," << e.datasizes[1] << ","
              << e.timers[0] << "," << e.timers[1] << "," << e.timers[2] << "," << e.timers[3] << std::endl;
  if (e.mode() == MODE_FULL) {
    timing_file << name << "," << e.current_id << "," << e.chunk_size() << "," << "0.0" << "," << "0.0" << ","
                << e.timers[3] << std::endl;
    size_file << name << "," << e.current_id << "," << e.chunk_size() << "," << e.datasizes[0] << ","
              << "0," << "0," << "0," << "0";
    for (uint32_t j = 0; j < e.current_id; j++) size_file << ",0";
    size_file << std::endl;
    return;
  }
  timing_file << name << "," << e.current_id << "," << e.chunk_size() << "," << e.timers[1] << "," << e.timers[2]
              << "," << e.timers[3] << std::endl;
  size_file << name << "," << e.current_id << "," << e.chunk_size() << "," << e.datasizes[0] << ","
            << e.datasizes[1] << ",";
  const uint32_t num_chkpts = e.mode() == MODE_BASIC ? e.current_id - e.baseline_id + 1 : e.current_id;
  write_metadata_breakdown(size_file, header, diff, diff_len, num_chkpts);
}

void write_restart_log(const Engine& e, uint32_t select_chkpt, const std::string& logname) {
  std::fstream timing_file;
  timing_file.open(logname, std::fstream::out | std::fstream::app);
  timing_file << approach_name(e.mode()) << ",";
  timing_file << select_chkpt << "," << e.chunk_size() << "," << e.restart_timers[0] << "," << e.restart_timers[1]
              << std::endl;
}

}  // namespace mtc
