// snapshot.cpp -- FLSHVEC1 snapshot files (see snapshot.h): a read-only
// memory map with the reference's validation, a small JSON reader for the
// manifest, and the writer.
#include "snapshot.h"

#include <errno.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>

#include "../../include/fv_bridge.h"

namespace fv {
namespace snap {

namespace {

constexpr char kMagic[8] = {'F', 'L', 'S', 'H', 'V', 'E', 'C', '1'};
constexpr uint64_t kAlign = 64;

uint64_t align_up(uint64_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// ------------------------------------------------------------------ JSON
// A JSON value: enough of the grammar for the manifest (objects, arrays,
// strings with escapes, numbers, true / false / null).
struct Value {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0.0;
  bool integral = false;
  uint64_t u = 0;  // exact value of a non-negative integer literal
  std::string s;
  std::vector<Value> arr;
  std::vector<std::pair<std::string, Value>> obj;
  const Value* get(const char* key) const {
    for (const auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
};

class Parser {
 public:
  Parser(const std::string& t) : t_(t) {}
  bool parse(Value* v) {
    ws();
    if (!value(v, 0)) return false;
    ws();
    return i_ == t_.size();
  }
  std::string error() const { return "manifest JSON: syntax error at byte " + std::to_string(i_); }

 private:
  void ws() {
    while (i_ < t_.size() && (t_[i_] == ' ' || t_[i_] == '\t' || t_[i_] == '\n' || t_[i_] == '\r')) ++i_;
  }
  bool lit(const char* w) {
    const size_t n = std::strlen(w);
    if (t_.compare(i_, n, w) != 0) return false;
    i_ += n;
    return true;
  }
  bool value(Value* v, int depth) {
    if (depth > 64 || i_ >= t_.size()) return false;
    const char c = t_[i_];
    if (c == '{') return object(v, depth);
    if (c == '[') return array(v, depth);
    if (c == '"') {
      v->kind = Value::String;
      return string(&v->s);
    }
    if (lit("true")) {
      v->kind = Value::Bool;
      v->b = true;
      return true;
    }
    if (lit("false")) {
      v->kind = Value::Bool;
      return true;
    }
    if (lit("null")) return true;
    return number(v);
  }
  bool object(Value* v, int depth) {
    v->kind = Value::Object;
    ++i_;
    ws();
    if (i_ < t_.size() && t_[i_] == '}') {
      ++i_;
      return true;
    }
    while (true) {
      ws();
      std::string key;
      if (i_ >= t_.size() || t_[i_] != '"' || !string(&key)) return false;
      ws();
      if (i_ >= t_.size() || t_[i_] != ':') return false;
      ++i_;
      ws();
      Value child;
      if (!value(&child, depth + 1)) return false;
      v->obj.emplace_back(std::move(key), std::move(child));
      ws();
      if (i_ < t_.size() && t_[i_] == ',') {
        ++i_;
        continue;
      }
      if (i_ < t_.size() && t_[i_] == '}') {
        ++i_;
        return true;
      }
      return false;
    }
  }
  bool array(Value* v, int depth) {
    v->kind = Value::Array;
    ++i_;
    ws();
    if (i_ < t_.size() && t_[i_] == ']') {
      ++i_;
      return true;
    }
    while (true) {
      ws();
      Value child;
      if (!value(&child, depth + 1)) return false;
      v->arr.push_back(std::move(child));
      ws();
      if (i_ < t_.size() && t_[i_] == ',') {
        ++i_;
        continue;
      }
      if (i_ < t_.size() && t_[i_] == ']') {
        ++i_;
        return true;
      }
      return false;
    }
  }
  bool string(std::string* out) {
    ++i_;  // opening quote
    while (i_ < t_.size()) {
      const char c = t_[i_++];
      if (c == '"') return true;
      if (c != '\\') {
        out->push_back(c);
        continue;
      }
      if (i_ >= t_.size()) return false;
      const char e = t_[i_++];
      switch (e) {
        case '"': out->push_back('"'); break;
        case '\\': out->push_back('\\'); break;
        case '/': out->push_back('/'); break;
        case 'b': out->push_back('\b'); break;
        case 'f': out->push_back('\f'); break;
        case 'n': out->push_back('\n'); break;
        case 'r': out->push_back('\r'); break;
        case 't': out->push_back('\t'); break;
        case 'u': {
          if (i_ + 4 > t_.size()) return false;
          unsigned cp = 0;
          for (int k = 0; k < 4; ++k) {
            const char h = t_[i_++];
            cp <<= 4;
            if (h >= '0' && h <= '9') cp |= (unsigned)(h - '0');
            else if (h >= 'a' && h <= 'f') cp |= (unsigned)(h - 'a' + 10);
            else if (h >= 'A' && h <= 'F') cp |= (unsigned)(h - 'A' + 10);
            else return false;
          }
          // section names are ASCII; other code points are kept as UTF-8
          if (cp < 0x80) {
            out->push_back((char)cp);
          } else if (cp < 0x800) {
            out->push_back((char)(0xC0 | (cp >> 6)));
            out->push_back((char)(0x80 | (cp & 0x3F)));
          } else {
            out->push_back((char)(0xE0 | (cp >> 12)));
            out->push_back((char)(0x80 | ((cp >> 6) & 0x3F)));
            out->push_back((char)(0x80 | (cp & 0x3F)));
          }
          break;
        }
        default: return false;
      }
    }
    return false;
  }
  bool number(Value* v) {
    const size_t start = i_;
    if (i_ < t_.size() && t_[i_] == '-') ++i_;
    bool digits = false, frac = false;
    while (i_ < t_.size() && t_[i_] >= '0' && t_[i_] <= '9') {
      ++i_;
      digits = true;
    }
    if (i_ < t_.size() && t_[i_] == '.') {
      frac = true;
      ++i_;
      while (i_ < t_.size() && t_[i_] >= '0' && t_[i_] <= '9') ++i_;
    }
    if (i_ < t_.size() && (t_[i_] == 'e' || t_[i_] == 'E')) {
      frac = true;
      ++i_;
      if (i_ < t_.size() && (t_[i_] == '+' || t_[i_] == '-')) ++i_;
      while (i_ < t_.size() && t_[i_] >= '0' && t_[i_] <= '9') ++i_;
    }
    if (!digits) return false;
    const std::string lit_s = t_.substr(start, i_ - start);
    v->kind = Value::Number;
    v->num = std::strtod(lit_s.c_str(), nullptr);
    v->integral = !frac && lit_s[0] != '-';
    if (v->integral) v->u = std::strtoull(lit_s.c_str(), nullptr, 10);
    return true;
  }
  const std::string& t_;
  size_t i_ = 0;
};

bool get_u64(const Value& o, const char* key, uint64_t* out, bool required, std::string* err) {
  const Value* v = o.get(key);
  if (!v) {
    if (required && err) *err = std::string("manifest: missing field ") + key;
    return !required;
  }
  if (v->kind != Value::Number || !v->integral) {
    if (err) *err = std::string("manifest: field ") + key + " is not a non-negative integer";
    return false;
  }
  *out = v->u;
  return true;
}

bool get_u32(const Value& o, const char* key, uint32_t* out, bool required, std::string* err) {
  uint64_t x = *out;
  if (!get_u64(o, key, &x, required, err)) return false;
  if (x > 0xFFFFFFFFull) {
    if (err) *err = std::string("manifest: field ") + key + " above u32";
    return false;
  }
  *out = (uint32_t)x;
  return true;
}

std::string json_string(const std::string& s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') {
      o.push_back('\\');
      o.push_back(c);
    } else if ((unsigned char)c < 0x20) {
      char b[8];
      std::snprintf(b, sizeof b, "\\u%04x", (unsigned)(unsigned char)c);
      o += b;
    } else {
      o.push_back(c);
    }
  }
  return o + "\"";
}

}  // namespace

int parse_manifest(const std::string& json, Manifest* out, std::string* error) {
  Value root;
  Parser p(json);
  if (!p.parse(&root) || root.kind != Value::Object) {
    if (error) *error = p.error();
    return FV_ERR_ARG;
  }
  Manifest m;
  const Value* cfg = root.get("config");
  if (!cfg || cfg->kind != Value::Object) {
    if (error) *error = "manifest: missing config object";
    return FV_ERR_ARG;
  }
  bool ok = get_u32(root, "version", &m.version, true, error) && get_u32(*cfg, "dim", &m.dim, true, error) &&
            get_u32(*cfg, "max_elements", &m.max_elements, false, error) && get_u32(*cfg, "m", &m.m, false, error) &&
            get_u32(*cfg, "ef_construction", &m.ef_construction, false, error) &&
            get_u32(*cfg, "nlist", &m.nlist, true, error) && get_u32(*cfg, "m_pq", &m.m_pq, true, error) &&
            get_u32(*cfg, "metric", &m.metric, true, error) &&
            get_u64(root, "num_vectors", &m.num_vectors, true, error) &&
            get_u32(root, "entry_point", &m.entry_point, false, error) &&
            get_u64(root, "cagra_degree", &m.cagra_degree, false, error) &&
            get_u64(root, "rabitq_padded_dim", &m.rabitq_padded_dim, false, error) &&
            get_u64(root, "fp16_padded_dim", &m.fp16_padded_dim, false, error) &&
            get_u64(root, "sparse_num_docs", &m.sparse_num_docs, false, error) &&
            get_u64(root, "sparse_nnz", &m.sparse_nnz, false, error) &&
            get_u32(root, "next_logical_id", &m.next_logical_id, true, error);
  if (!ok) return FV_ERR_ARG;
  if (const Value* seeds = root.get("cagra_seeds")) {
    for (const Value& s : seeds->arr) m.cagra_seeds.push_back((uint32_t)s.u);
  }
  const Value* secs = root.get("sections");
  if (!secs || secs->kind != Value::Object) {
    if (error) *error = "manifest: missing sections object";
    return FV_ERR_ARG;
  }
  for (const auto& kv : secs->obj) {
    Section s;
    const Value& v = kv.second;
    if (v.kind != Value::Object || !get_u64(v, "offset", &s.offset, true, error) ||
        !get_u64(v, "byte_len", &s.byte_len, true, error) || !get_u64(v, "len", &s.len, true, error))
      return FV_ERR_ARG;
    const Value* dt = v.get("dtype");
    if (!dt || dt->kind != Value::String) {
      if (error) *error = "manifest: section " + kv.first + " has no dtype";
      return FV_ERR_ARG;
    }
    s.dtype = dt->s;
    m.sections[kv.first] = s;
  }
  *out = std::move(m);
  return 0;
}

std::string manifest_to_json(const Manifest& m) {
  std::string o = "{\"version\":" + std::to_string(m.version) + ",\"config\":{\"dim\":" + std::to_string(m.dim) +
                  ",\"max_elements\":" + std::to_string(m.max_elements) + ",\"m\":" + std::to_string(m.m) +
                  ",\"ef_construction\":" + std::to_string(m.ef_construction) + ",\"nlist\":" +
                  std::to_string(m.nlist) + ",\"m_pq\":" + std::to_string(m.m_pq) + ",\"metric\":" +
                  std::to_string(m.metric) + "},\"num_vectors\":" + std::to_string(m.num_vectors) +
                  ",\"entry_point\":" + std::to_string(m.entry_point) + ",\"cagra_degree\":" +
                  std::to_string(m.cagra_degree) + ",\"cagra_seeds\":[";
  for (size_t i = 0; i < m.cagra_seeds.size(); ++i) o += (i ? "," : "") + std::to_string(m.cagra_seeds[i]);
  o += "],\"rabitq_padded_dim\":" + std::to_string(m.rabitq_padded_dim) +
       ",\"fp16_padded_dim\":" + std::to_string(m.fp16_padded_dim) +
       ",\"sparse_num_docs\":" + std::to_string(m.sparse_num_docs) + ",\"sparse_nnz\":" +
       std::to_string(m.sparse_nnz) + ",\"next_logical_id\":" + std::to_string(m.next_logical_id) +
       ",\"sections\":{";
  bool first = true;
  for (const auto& kv : m.sections) {
    if (!first) o += ",";
    first = false;
    o += json_string(kv.first) + ":{\"offset\":" + std::to_string(kv.second.offset) +
         ",\"byte_len\":" + std::to_string(kv.second.byte_len) + ",\"dtype\":" + json_string(kv.second.dtype) +
         ",\"len\":" + std::to_string(kv.second.len) + "}";
  }
  return o + "}}";
}

// ------------------------------------------------------------------ File
File::~File() {
  if (map_) munmap(map_, size_);
}

int File::open(const char* path, std::string* error) {
  const int fd = ::open(path, O_RDONLY | O_CLOEXEC);
  if (fd < 0) {
    if (error) *error = std::string("open ") + path + ": " + std::strerror(errno);
    return -100 - errno;
  }
  struct stat st;
  if (fstat(fd, &st) != 0) {
    const int e = errno;
    ::close(fd);
    if (error) *error = std::string("stat ") + path + ": " + std::strerror(e);
    return -100 - e;
  }
  size_ = (size_t)st.st_size;
  if (size_ < 16) {
    ::close(fd);
    if (error) *error = "snapshot shorter than its 16-byte header";
    return FV_ERR_ARG;
  }
  map_ = mmap(nullptr, size_, PROT_READ, MAP_SHARED, fd, 0);
  const int e = errno;
  ::close(fd);
  if (map_ == MAP_FAILED) {
    map_ = nullptr;
    if (error) *error = std::string("mmap: ") + std::strerror(e);
    return -100 - e;
  }
  const uint8_t* b = base();
  if (std::memcmp(b, kMagic, 8) != 0) {
    if (error) *error = "invalid snapshot magic header";
    return FV_ERR_ARG;
  }
  uint64_t hlen = 0;
  for (int i = 7; i >= 0; --i) hlen = (hlen << 8) | b[8 + i];  // little endian
  if (hlen > size_ - 16) {
    if (error) *error = "truncated snapshot header";
    return FV_ERR_ARG;
  }
  json_.assign(reinterpret_cast<const char*>(b + 16), (size_t)hlen);
  int rc = parse_manifest(json_, &m_, error);
  if (rc) return rc;
  data_start_ = align_up(16 + hlen);
  if (data_start_ > size_ && !m_.sections.empty()) {
    if (error) *error = "truncated snapshot payload";
    return FV_ERR_ARG;
  }
  for (const auto& kv : m_.sections) {
    const uint64_t end = data_start_ + kv.second.offset + kv.second.byte_len;
    if (end < data_start_ || end > size_) {
      if (error) *error = "truncated section: " + kv.first;
      return FV_ERR_ARG;
    }
  }
  return 0;
}

const uint8_t* File::section(const char* name, uint64_t* bytes) const {
  auto it = m_.sections.find(name);
  if (it == m_.sections.end()) {
    if (bytes) *bytes = 0;
    return nullptr;
  }
  if (bytes) *bytes = it->second.byte_len;
  return base() + data_start_ + it->second.offset;
}

int write(const char* path, Manifest m, const std::vector<OutSection>& sections, std::string* error) {
  uint64_t cursor = 0;
  m.sections.clear();
  for (const auto& s : sections) {
    cursor = align_up(cursor);
    Section meta;
    meta.offset = cursor;
    meta.byte_len = s.bytes;
    meta.dtype = s.dtype;
    meta.len = s.len;
    m.sections[s.name] = meta;
    cursor += s.bytes;
  }
  const std::string json = manifest_to_json(m);
  std::unique_ptr<FILE, int (*)(FILE*)> f(std::fopen(path, "wb"), &std::fclose);
  if (!f) {
    if (error) *error = std::string("create snapshot ") + path + ": " + std::strerror(errno);
    return -100 - errno;
  }
  uint8_t head[16];
  std::memcpy(head, kMagic, 8);
  const uint64_t hlen = json.size();
  for (int i = 0; i < 8; ++i) head[8 + i] = (uint8_t)(hlen >> (8 * i));
  const uint64_t data_start = align_up(16 + hlen);
  static const uint8_t zeros[kAlign] = {};
  bool ok = std::fwrite(head, 1, 16, f.get()) == 16 && std::fwrite(json.data(), 1, json.size(), f.get()) == json.size();
  if (ok && data_start > 16 + hlen) ok = std::fwrite(zeros, 1, data_start - 16 - hlen, f.get()) == data_start - 16 - hlen;
  uint64_t written = 0;
  for (const auto& s : sections) {
    if (!ok) break;
    const uint64_t aligned = align_up(written);
    if (aligned > written) ok = std::fwrite(zeros, 1, aligned - written, f.get()) == aligned - written;
    written = aligned;
    if (ok && s.bytes) ok = std::fwrite(s.data, 1, s.bytes, f.get()) == s.bytes;
    written += s.bytes;
  }
  if (!ok || std::fflush(f.get()) != 0) {
    if (error) *error = std::string("write snapshot: ") + std::strerror(errno);
    return -100 - errno;
  }
  return 0;
}

}  // namespace snap
}  // namespace fv
