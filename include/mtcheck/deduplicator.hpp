// mtcheck/deduplicator.hpp -- C++ interface of the GB300 deduplicator with the
// class names, overloads and behaviour of the reference's BaseDeduplicator
// (include/deduplicator_interface.hpp:14-184) and its four subclasses.
//
// Header-only, over the C ABI of <mtcheck.h>.  The reference's Kokkos types
// are replaced by plain ones:
//   Kokkos::View<uint8_t*> data           -> uint8_t* device pointer + length
//   Kokkos::View<uint8_t*>::HostMirror    -> std::vector<uint8_t>
//   std::vector<HostMirror> chkpts        -> std::vector<std::vector<uint8_t>>
// Failures throw mtcheck::Error (the reference throws std::ifstream /
// std::ofstream exceptions on file errors and prints everything else).
#ifndef MTCHECK_DEDUPLICATOR_HPP
#define MTCHECK_DEDUPLICATOR_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../mtcheck.h"

namespace mtcheck {

using header_t = mtc_header_t;  // include/utils.hpp:29-37

// DedupMode, include/utils.hpp:39-49
enum DedupMode { Unknown = 0, Full = MTC_FULL, Basic = MTC_BASIC, List = MTC_LIST, Tree = MTC_TREE,
                 TreeLowOffsetRef = MTC_TREE_LOW_OFFSET_REF, TreeLowOffset = MTC_TREE_LOW_OFFSET };
enum HashKind { Murmur3 = MTC_HASH_MURMUR3, MD5 = MTC_HASH_MD5 };

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc != MTC_OK) throw Error(rc, mtc_last_error());
}

class BaseDeduplicator {
 protected:
  mtc_dedup_t* h_ = nullptr;
  uint32_t chunk_size;
  int mode_;

  BaseDeduplicator(int mode, uint32_t bytes_per_chunk, HashKind hash)
      : chunk_size(bytes_per_chunk), mode_(mode) {
    check(mtc_create(mode, hash, bytes_per_chunk, &h_));
  }

  static const char* suffix(int mode) {  // src/dedup_files.cpp:87-99
    switch (mode) {
      case MTC_FULL: return ".full_chkpt";
      case MTC_BASIC: return ".basic.incr_chkpt";
      case MTC_LIST: return ".hashlist.incr_chkpt";
      default: return ".hashtree.incr_chkpt";
    }
  }
  static void host_chain(std::vector<std::vector<uint8_t>>& chkpts, std::vector<const void*>& p,
                         std::vector<uint64_t>& l) {
    for (auto& c : chkpts) {
      p.push_back(c.data());
      l.push_back(c.size());
    }
  }

 public:
  BaseDeduplicator(const BaseDeduplicator&) = delete;
  BaseDeduplicator& operator=(const BaseDeduplicator&) = delete;
  virtual ~BaseDeduplicator() { mtc_destroy(h_); }

  // checkpoint(header_t&, uint8_t*, size_t, HostMirror&, bool), :52-57
  void checkpoint(header_t& header, uint8_t* data_ptr, size_t data_len, std::vector<uint8_t>& diff_h,
                  bool make_baseline) {
    uint64_t n = 0;
    check(mtc_checkpoint_header(h_, &header, data_ptr, data_len, make_baseline ? 1 : 0, &n));
    diff_h.resize(n);
    check(mtc_diff_copy(h_, diff_h.data(), n));
  }
  // checkpoint(uint8_t*, size_t, std::string& filename, std::string& logname, bool), :73-77
  void checkpoint(uint8_t* data_ptr, size_t len, std::string& filename, std::string& logname, bool make_baseline) {
    check(mtc_checkpoint_file(h_, data_ptr, len, filename.c_str(), logname.c_str(), make_baseline ? 1 : 0));
  }
  // checkpoint(uint8_t*, size_t, HostMirror&, bool), :93-96
  void checkpoint(uint8_t* data_ptr, size_t len, std::vector<uint8_t>& diff_h, bool make_baseline) {
    header_t header;
    checkpoint(header, data_ptr, len, diff_h, make_baseline);
    check(mtc_advance(h_));
  }
  // checkpoint(uint8_t*, size_t, HostMirror&, std::string& logname, bool), :113-117
  void checkpoint(uint8_t* data_ptr, size_t len, std::vector<uint8_t>& diff_h, std::string& logname,
                  bool make_baseline) {
    header_t header;
    checkpoint(header, data_ptr, len, diff_h, make_baseline);
    write_chkpt_log(header, diff_h, logname);
    check(mtc_advance(h_));
  }

  // restart(uint8_t*, size_t, std::vector<HostMirror>&, std::string& logname, uint32_t), :142-146;
  // writes <logname>.chunk_size.<c>.restart_timing.csv like the reference
  void restart(uint8_t* data_ptr, size_t len, std::vector<std::vector<uint8_t>>& chkpts, std::string& logname,
               uint32_t chkpt_id) {
    std::vector<const void*> p;
    std::vector<uint64_t> l;
    host_chain(chkpts, p, l);
    check(mtc_restart(h_, data_ptr, len, p.data(), l.data(), (uint32_t)p.size(), chkpt_id));
    std::string log = logname + ".chunk_size." + std::to_string(chunk_size) + ".restart_timing.csv";
    write_restart_log(chkpt_id, log);
  }
  // restart(View, std::vector<std::string>& chkpt_filenames, std::string& logname, uint32_t), :156-159:
  // the approach's suffix is appended to every name (src/tree_approach.cpp:1832-1835)
  void restart(uint8_t* data_ptr, size_t len, std::vector<std::string>& chkpt_filenames, std::string& logname,
               uint32_t chkpt_id) {
    std::vector<std::string> names;
    std::vector<const char*> p;
    for (auto& f : chkpt_filenames) names.push_back(f + suffix(mode_));
    for (auto& f : names) p.push_back(f.c_str());
    check(mtc_restart_files(h_, data_ptr, len, p.data(), (uint32_t)p.size(), chkpt_id));
    write_restart_log(chkpt_id, logname);
  }
  // the restart with the chain already in device memory (no reference counterpart)
  void restart_device(uint8_t* data_ptr, size_t len, const std::vector<std::pair<const uint8_t*, uint64_t>>& chain,
                      uint32_t chkpt_id) {
    std::vector<const void*> p;
    std::vector<uint64_t> l;
    for (auto& c : chain) {
      p.push_back(c.first);
      l.push_back(c.second);
    }
    check(mtc_restart_device(h_, data_ptr, len, p.data(), l.data(), (uint32_t)p.size(), chkpt_id));
  }
  // frees the restart tables the handle keeps between restarts (no reference counterpart)
  void release_restart_buffers() { check(mtc_release_restart_buffers(h_)); }

  // write_chkpt_log / write_restart_log, :172-183
  void write_chkpt_log(header_t& header, std::vector<uint8_t>& diff_h, std::string& logname) {
    check(mtc_write_chkpt_log(h_, &header, diff_h.data(), diff_h.size(), logname.c_str()));
  }
  void write_restart_log(uint32_t select_chkpt, std::string& logname) {
    check(mtc_write_restart_log(h_, select_chkpt, logname.c_str()));
  }

  mtc_info_t info() const {
    mtc_info_t i;
    check(mtc_get_info(h_, &i));
    return i;
  }
  uint32_t current_id() const { return info().current_id; }
  void set_stream(void* cuda_stream) { check(mtc_set_stream(h_, cuda_stream)); }
  mtc_dedup_t* handle() { return h_; }
};

class FullDeduplicator : public BaseDeduplicator {
 public:
  explicit FullDeduplicator(uint32_t bytes_per_chunk, HashKind hash = Murmur3)
      : BaseDeduplicator(MTC_FULL, bytes_per_chunk, hash) {}
};
class BasicDeduplicator : public BaseDeduplicator {
 public:
  explicit BasicDeduplicator(uint32_t bytes_per_chunk, HashKind hash = Murmur3)
      : BaseDeduplicator(MTC_BASIC, bytes_per_chunk, hash) {}
};
class ListDeduplicator : public BaseDeduplicator {
 public:
  explicit ListDeduplicator(uint32_t bytes_per_chunk, HashKind hash = Murmur3)
      : BaseDeduplicator(MTC_LIST, bytes_per_chunk, hash) {}
  size_t num_first_ocur() const { return info().num_first_ocur; }
  size_t num_shift_dupl() const { return info().num_shift_dupl; }
};
// TreeDeduplicator, include/tree_approach.hpp:16-205
class TreeDeduplicator : public BaseDeduplicator {
 public:
  explicit TreeDeduplicator(uint32_t bytes_per_chunk, HashKind hash = Murmur3, int mode = MTC_TREE)
      : BaseDeduplicator(mode, bytes_per_chunk, hash) {}
  size_t num_first_ocur() const { return info().num_first_ocur; }  // :52-54
  size_t num_shift_dupl() const { return info().num_shift_dupl; }  // :56-58
};

}  // namespace mtcheck
#endif  // MTCHECK_DEDUPLICATOR_HPP
