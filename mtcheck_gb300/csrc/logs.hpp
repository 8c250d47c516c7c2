// logs.hpp -- the CSV logs of the reference: write_chkpt_log
// (src/tree_approach.cpp:1854-1896 and siblings), write_metadata_breakdown
// (src/utils.cpp:38-124) and write_restart_log (src/tree_approach.cpp:1905-1915).
#pragma once
#include <cstdint>
#include <string>

#include "engine.hpp"

namespace mtc {
void write_chkpt_log(const Engine& e, const HeaderHost& header, const uint8_t* diff, uint64_t diff_len,
                     const std::string& logname);
void write_restart_log(const Engine& e, uint32_t select_chkpt, const std::string& logname);
}
