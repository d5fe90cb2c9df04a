// snapshot.h -- the reference's FLSHVEC1 snapshot file (persistence.rs:1-200):
//   [0, 8)          magic "FLSHVEC1"
//   [8, 16)         little-endian u64 length H of the JSON manifest
//   [16, 16 + H)    UTF-8 JSON manifest (config, counts, section table)
//   [data_start, )  data_start = 16 + H rounded up to 64; every section at
//                   data_start + offset, offsets multiples of 64
// Host code only (no CUDA): the engine (engine.cpp) maps sections into its
// device tables.
#pragma once

#include <stdint.h>

#include <map>
#include <string>
#include <vector>

namespace fv {
namespace snap {

struct Section {
  uint64_t offset = 0, byte_len = 0, len = 0;
  std::string dtype;
};

// SnapshotManifest (persistence.rs:35-49) with IndexConfig (ffi.rs:122-130).
struct Manifest {
  uint32_t version = 1;
  uint32_t dim = 0, max_elements = 0, m = 32, ef_construction = 128, nlist = 0, m_pq = 0, metric = 0;
  uint64_t num_vectors = 0;
  uint32_t entry_point = 0;
  uint64_t cagra_degree = 0;
  std::vector<uint32_t> cagra_seeds;
  uint64_t rabitq_padded_dim = 0, fp16_padded_dim = 0, sparse_num_docs = 0, sparse_nnz = 0;
  uint32_t next_logical_id = 0;
  std::map<std::string, Section> sections;
};

// Read-only memory map of a snapshot file, validated as MmapSnapshot::open
// does (persistence.rs:133-170): magic, header bounds, every section in range.
class File {
 public:
  File() = default;
  ~File();
  File(const File&) = delete;
  File& operator=(const File&) = delete;
  // 0 on success, else FV_ERR_ARG (format) / an errno-derived code (< -100)
  int open(const char* path, std::string* error);
  const Manifest& manifest() const { return m_; }
  const std::string& manifest_json() const { return json_; }
  // bytes of a section (nullptr and 0 when absent)
  const uint8_t* section(const char* name, uint64_t* bytes) const;
  const uint8_t* base() const { return static_cast<const uint8_t*>(map_); }
  size_t size() const { return size_; }

 private:
  void* map_ = nullptr;
  size_t size_ = 0;
  uint64_t data_start_ = 0;
  Manifest m_;
  std::string json_;
};

// One section to write: name, dtype ("f32", "u32", "u16", "u8"), element
// count and the bytes.
struct OutSection {
  std::string name, dtype;
  uint64_t len;
  const void* data;
  uint64_t bytes;
};

// Writes a FLSHVEC1 file: manifest (its section table is filled in here)
// and sections in the order given, each 64-byte aligned (persistence.rs:52-110).
int write(const char* path, Manifest m, const std::vector<OutSection>& sections, std::string* error);

// Manifest <-> JSON (the field names and types serde uses for the
// reference's structs; unknown fields are ignored on read).
int parse_manifest(const std::string& json, Manifest* out, std::string* error);
std::string manifest_to_json(const Manifest& m);

}  // namespace snap
}  // namespace fv
