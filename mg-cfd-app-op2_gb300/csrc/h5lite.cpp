// h5lite: HDF5-subset reader/writer.  The supported subset and the reason it
// exists are described in h5lite.h.  Byte layouts follow the public HDF5 File
// Format Specification (superblock v0/v1, symbol-table groups, version-1
// B-trees, local heaps, version-1 object headers, dataspace/datatype/
// fill-value/layout/attribute messages).
#include "h5lite.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <set>

namespace h5lite {
namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kLeafK = 4;       // symbol-table node holds 2*kLeafK entries
constexpr int kInternalK = 16;  // group B-tree node holds 2*kInternalK children
constexpr uint64_t kHeapFreeNull = 1;  // "no free block" marker of local heaps

uint64_t pad8(uint64_t n) { return (n + 7) & ~7ull; }

class Out {
 public:
  std::vector<uint8_t> b;
  void u8(uint8_t v) { b.push_back(v); }
  void u16(uint16_t v) { put(&v, 2); }
  void u32(uint32_t v) { put(&v, 4); }
  void u64(uint64_t v) { put(&v, 8); }
  void put(const void* p, size_t n) {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    b.insert(b.end(), c, c + n);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void align8() { while (b.size() % 8) b.push_back(0); }
  size_t size() const { return b.size(); }
};

// ---- message encoders (each returns the message body, padded to 8) ---------

std::vector<uint8_t> msg_dataspace(int rank, const uint64_t* dims) {
  Out o;
  o.u8(1);                  // version
  o.u8((uint8_t)rank);
  o.u8(1);                  // flags: maximum dimensions present
  o.u8(0);
  o.u32(0);
  for (int i = 0; i < rank; i++) o.u64(dims[i]);
  for (int i = 0; i < rank; i++) o.u64(dims[i]);
  o.align8();
  return o.b;
}

std::vector<uint8_t> msg_datatype(DType t) {
  Out o;
  if (t == F64) {
    o.u8(0x11);             // version 1, class 1 (floating point)
    o.u8(0x20);             // little endian, mantissa normalisation "implied"
    o.u8(63);               // sign bit position
    o.u8(0);
    o.u32(8);
    o.u16(0);               // bit offset
    o.u16(64);              // bit precision
    o.u8(52);               // exponent location
    o.u8(11);               // exponent size
    o.u8(0);                // mantissa location
    o.u8(52);               // mantissa size
    o.u32(1023);            // exponent bias
  } else {
    o.u8(0x10);             // version 1, class 0 (fixed point)
    o.u8(0x08);             // little endian, signed
    o.u8(0);
    o.u8(0);
    o.u32(4);
    o.u16(0);
    o.u16(32);
  }
  o.align8();
  return o.b;
}

std::vector<uint8_t> msg_string_type(uint32_t len) {
  Out o;
  o.u8(0x13);               // version 1, class 3 (string)
  o.u8(0x00);               // null-terminated, ASCII
  o.u8(0);
  o.u8(0);
  o.u32(len);
  return o.b;               // 8 bytes, no properties
}

std::vector<uint8_t> msg_fill_value() {
  Out o;
  o.u8(2);                  // version 2
  o.u8(2);                  // space allocation time: late
  o.u8(2);                  // fill value write time: if set by user
  o.u8(0);                  // fill value undefined
  o.align8();
  return o.b;
}

std::vector<uint8_t> msg_layout_contiguous(uint64_t addr, uint64_t size) {
  Out o;
  o.u8(3);                  // version 3
  o.u8(1);                  // contiguous
  o.u64(addr);
  o.u64(size);
  o.align8();
  return o.b;
}

std::vector<uint8_t> msg_attribute(const std::string& name,
                                   const std::vector<uint8_t>& dtype,
                                   const void* value, size_t value_size) {
  Out o;
  uint64_t one = 1;
  std::vector<uint8_t> space;
  {
    Out s;
    s.u8(1); s.u8(1); s.u8(0); s.u8(0); s.u32(0); s.u64(one);
    space = s.b;
  }
  o.u8(1);                  // version 1
  o.u8(0);
  o.u16((uint16_t)(name.size() + 1));
  o.u16((uint16_t)dtype.size());
  o.u16((uint16_t)space.size());
  o.put(name.c_str(), name.size() + 1);
  o.align8();
  o.put(dtype.data(), dtype.size());
  o.align8();
  o.put(space.data(), space.size());
  o.align8();
  o.put(value, value_size);
  o.align8();
  return o.b;
}

struct Msg { uint16_t type; std::vector<uint8_t> body; };

uint64_t object_header_size(const std::vector<Msg>& msgs) {
  uint64_t n = 16;
  for (auto& m : msgs) n += 8 + m.body.size();
  return n;
}

void emit_object_header(Out& o, const std::vector<Msg>& msgs) {
  uint64_t body = object_header_size(msgs) - 16;
  o.u8(1);                  // version 1
  o.u8(0);
  o.u16((uint16_t)msgs.size());
  o.u32(1);                 // reference count
  o.u32((uint32_t)body);
  o.u32(0);                 // pad prefix to 16 bytes
  for (auto& m : msgs) {
    o.u16(m.type);
    o.u16((uint16_t)m.body.size());
    o.u8(0);
    o.u8(0); o.u8(0); o.u8(0);
    o.put(m.body.data(), m.body.size());
  }
}

std::vector<Msg> dataset_messages(const DatasetOut& d, uint64_t data_addr) {
  uint64_t dims[2] = {d.rows, d.cols};
  int rank = d.cols == 0 ? 1 : 2;
  uint64_t esize = d.dtype == F64 ? 8 : 4;
  uint64_t nbytes = d.rows * (d.cols ? d.cols : 1) * esize;
  std::vector<Msg> m;
  m.push_back({0x0001, msg_dataspace(rank, dims)});
  m.push_back({0x0003, msg_datatype(d.dtype)});
  m.push_back({0x0005, msg_fill_value()});
  m.push_back({0x0008, msg_layout_contiguous(nbytes ? data_addr : kUndef, nbytes)});
  if (d.op2_attributes) {
    int32_t dim = (int32_t)(d.cols ? d.cols : 1);
    int32_t size = (int32_t)(dim * esize);
    std::vector<uint8_t> ityp = msg_datatype(I32);
    m.push_back({0x000C, msg_attribute("dim", ityp, &dim, 4)});
    m.push_back({0x000C, msg_attribute("size", ityp, &size, 4)});
    char tname[10] = {0};
    std::strncpy(tname, d.dtype == F64 ? "double" : "int", sizeof(tname) - 1);
    m.push_back({0x000C, msg_attribute("type", msg_string_type(10), tname, 10)});
  }
  return m;
}

}  // namespace

bool write_file(const std::string& path, const std::vector<DatasetOut>& sets_in,
                std::string* err) {
  std::vector<DatasetOut> sets = sets_in;
  std::sort(sets.begin(), sets.end(),
            [](const DatasetOut& a, const DatasetOut& b) { return std::strcmp(a.name.c_str(), b.name.c_str()) < 0; });
  for (size_t i = 1; i < sets.size(); i++)
    if (sets[i].name == sets[i - 1].name) { *err = "duplicate dataset name " + sets[i].name; return false; }
  const size_t per_snod = 2 * kLeafK;
  size_t n_snod = (sets.size() + per_snod - 1) / per_snod;
  if (n_snod == 0) n_snod = 1;
  if (n_snod > 2 * (size_t)kInternalK) { *err = "too many datasets for one group B-tree node"; return false; }

  // Local heap data segment: "" at offset 0, then each name.
  Out heap;
  heap.zeros(8);
  std::vector<uint64_t> name_off(sets.size());
  for (size_t i = 0; i < sets.size(); i++) {
    name_off[i] = heap.size();
    heap.put(sets[i].name.c_str(), sets[i].name.size() + 1);
    heap.align8();
  }

  // Fixed-size regions.
  const uint64_t sb_size = 96;
  std::vector<Msg> root_msgs = {{0x0011, std::vector<uint8_t>(16, 0)}};
  const uint64_t root_oh_addr = sb_size;
  const uint64_t root_oh_size = object_header_size(root_msgs);
  const uint64_t heap_hdr_addr = root_oh_addr + root_oh_size;
  const uint64_t heap_data_addr = heap_hdr_addr + 32;
  const uint64_t btree_addr = heap_data_addr + heap.size();
  const uint64_t btree_size = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
  const uint64_t snod_size = 8 + 2 * kLeafK * 40;
  const uint64_t snod_addr0 = btree_addr + btree_size;
  uint64_t cursor = snod_addr0 + n_snod * snod_size;

  std::vector<uint64_t> oh_addr(sets.size()), data_addr(sets.size()), data_size(sets.size());
  for (size_t i = 0; i < sets.size(); i++) {
    const DatasetOut& d = sets[i];
    uint64_t esize = d.dtype == F64 ? 8 : 4;
    data_size[i] = d.rows * (d.cols ? d.cols : 1) * esize;
    oh_addr[i] = cursor;
    cursor += object_header_size(dataset_messages(d, 0));
    cursor = pad8(cursor);
    data_addr[i] = cursor;
    cursor = pad8(cursor + data_size[i]);
  }
  const uint64_t eof = cursor;

  Out o;
  // Superblock version 0.
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  o.put(sig, 8);
  o.u8(0); o.u8(0); o.u8(0); o.u8(0); o.u8(0);
  o.u8(8); o.u8(8); o.u8(0);
  o.u16(kLeafK); o.u16(kInternalK);
  o.u32(0);
  o.u64(0);            // base address
  o.u64(kUndef);       // free-space info
  o.u64(eof);          // end of file
  o.u64(kUndef);       // driver info
  o.u64(0);            // root entry: link name offset
  o.u64(root_oh_addr);
  o.u32(1);            // cache type: symbol table
  o.u32(0);
  o.u64(btree_addr);
  o.u64(heap_hdr_addr);
  // Root object header with the symbol table message.
  {
    Out st; st.u64(btree_addr); st.u64(heap_hdr_addr);
    root_msgs[0].body = st.b;
    emit_object_header(o, root_msgs);
  }
  // Local heap.
  o.put("HEAP", 4); o.u8(0); o.u8(0); o.u8(0); o.u8(0);
  o.u64(heap.size());
  o.u64(kHeapFreeNull);
  o.u64(heap_data_addr);
  o.put(heap.b.data(), heap.size());
  // Group B-tree leaf node pointing at the symbol-table nodes.
  {
    size_t start = o.size();
    o.put("TREE", 4); o.u8(0); o.u8(0); o.u16((uint16_t)n_snod);
    o.u64(kUndef); o.u64(kUndef);
    o.u64(0);  // key 0: empty name
    for (size_t s = 0; s < n_snod; s++) {
      o.u64(snod_addr0 + s * snod_size);
      size_t last = std::min(sets.size(), (s + 1) * per_snod);
      o.u64(sets.empty() ? 0 : name_off[last - 1]);
    }
    o.zeros(btree_size - (o.size() - start));
  }
  for (size_t s = 0; s < n_snod; s++) {
    size_t start = o.size();
    size_t first = s * per_snod, last = std::min(sets.size(), (s + 1) * per_snod);
    o.put("SNOD", 4); o.u8(1); o.u8(0); o.u16((uint16_t)(last > first ? last - first : 0));
    for (size_t i = first; i < last; i++) {
      o.u64(name_off[i]); o.u64(oh_addr[i]); o.u32(0); o.u32(0); o.zeros(16);
    }
    o.zeros(snod_size - (o.size() - start));
  }
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { *err = "cannot create " + path; return false; }
  bool ok = std::fwrite(o.b.data(), 1, o.size(), f) == o.size();
  uint64_t pos = o.size();
  for (size_t i = 0; i < sets.size() && ok; i++) {
    Out h;
    emit_object_header(h, dataset_messages(sets[i], data_addr[i]));
    if (pos != oh_addr[i]) { ok = false; break; }
    ok = std::fwrite(h.b.data(), 1, h.size(), f) == h.size();
    pos += h.size();
    static const uint8_t zero8[8] = {0};
    while (ok && pos < data_addr[i]) { ok = std::fwrite(zero8, 1, 1, f) == 1; pos++; }
    if (ok && data_size[i]) ok = std::fwrite(sets[i].data, 1, data_size[i], f) == data_size[i];
    pos += data_size[i];
    while (ok && pos % 8) { ok = std::fwrite(zero8, 1, 1, f) == 1; pos++; }
  }
  ok = ok && pos == eof;
  if (std::fclose(f) != 0) ok = false;
  if (!ok) { *err = "write failed for " + path; return false; }
  return true;
}

// ---------------------------------------------------------------------------
// Reader
// ---------------------------------------------------------------------------
namespace {

struct Cursor {
  const std::vector<uint8_t>* b;
  uint64_t p;
  bool ok = true;
  bool need(uint64_t n) {
    if (!ok || p > b->size() || b->size() - p < n) { ok = false; return false; }
    return true;
  }
  uint64_t uN(int n) {
    if (!need(n)) return 0;
    uint64_t v = 0;
    std::memcpy(&v, b->data() + p, n);
    p += n;
    return v;
  }
  uint8_t u8() { return (uint8_t)uN(1); }
  uint16_t u16() { return (uint16_t)uN(2); }
  uint32_t u32() { return (uint32_t)uN(4); }
  uint64_t u64() { return uN(8); }
};

}  // namespace

bool File::open(const std::string& path, std::string* err) {
  sets_.clear();
  bytes_.clear();
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) { *err = "cannot open " + path; return false; }
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0) { std::fclose(f); *err = "cannot size " + path; return false; }
  bytes_.resize((size_t)sz);
  size_t got = sz ? std::fread(bytes_.data(), 1, (size_t)sz, f) : 0;
  std::fclose(f);
  if (got != (size_t)sz) { *err = "short read on " + path; return false; }

  static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  uint64_t sb = kUndef;
  for (uint64_t off = 0; off + 8 <= bytes_.size(); off = off ? off * 2 : 512) {
    if (std::memcmp(bytes_.data() + off, sig, 8) == 0) { sb = off; break; }
  }
  if (sb == kUndef) { *err = path + ": not an HDF5 file"; return false; }
  Cursor c{&bytes_, sb + 8};
  int sb_ver = c.u8();
  if (sb_ver > 1) { *err = path + ": HDF5 superblock version " + std::to_string(sb_ver) + " is not supported (only 0 and 1)"; return false; }
  c.u8(); c.u8(); c.u8(); c.u8();
  int so = c.u8(), sl = c.u8();
  if (so != 8 || sl != 8) { *err = path + ": only 8-byte offsets/lengths are supported"; return false; }
  c.u8();
  c.u16(); c.u16();
  c.u32();
  if (sb_ver == 1) { c.u16(); c.u16(); }
  base_ = c.u64();
  c.u64(); c.u64(); c.u64();
  c.u64();                         // root link name offset
  uint64_t root_oh = c.u64();
  uint32_t cache = c.u32();
  c.u32();
  uint64_t btree = c.u64(), heap = c.u64();
  if (!c.ok) { *err = path + ": truncated superblock"; return false; }

  // Object header walker shared by the root group and the datasets.
  auto walk_header = [&](uint64_t addr, const std::function<void(uint16_t, Cursor&, uint64_t)>& fn) -> bool {
    Cursor h{&bytes_, base_ + addr};
    int ver = h.u8();
    if (ver != 1) return false;
    h.u8();
    int nmsg = h.u16();
    h.u32();
    uint64_t size = h.u32();
    h.u32();
    std::vector<std::pair<uint64_t, uint64_t>> chunks = {{h.p, size}};
    int seen = 0;
    for (size_t ci = 0; ci < chunks.size() && ci < 64; ci++) {
      uint64_t p = chunks[ci].first, end = chunks[ci].first + chunks[ci].second;
      while (p + 8 <= end && seen < nmsg) {
        Cursor m{&bytes_, p};
        uint16_t type = m.u16();
        uint16_t msize = m.u16();
        m.u8(); m.u8(); m.u8(); m.u8();
        if (!m.ok || m.p + msize > end) return false;
        seen++;
        if (type == 0x0010) {
          Cursor cc{&bytes_, m.p};
          uint64_t off = cc.u64(), len = cc.u64();
          if (!cc.ok) return false;
          chunks.push_back({base_ + off, len});
        } else {
          Cursor body{&bytes_, m.p};
          fn(type, body, msize);
        }
        p = m.p + msize;
      }
    }
    return true;
  };

  bool have_st = false;
  walk_header(root_oh, [&](uint16_t type, Cursor& m, uint64_t) {
    if (type == 0x0011) { btree = m.u64(); heap = m.u64(); have_st = m.ok; }
  });
  if (!have_st && cache != 1) { *err = path + ": root group is not a symbol-table group (newer HDF5 format not supported)"; return false; }

  Cursor hh{&bytes_, base_ + heap};
  char hs[4];
  for (int i = 0; i < 4; i++) hs[i] = (char)hh.u8();
  if (std::memcmp(hs, "HEAP", 4) != 0) { *err = path + ": bad local heap"; return false; }
  hh.u8(); hh.u8(); hh.u8(); hh.u8();
  uint64_t heap_size = hh.u64();
  hh.u64();
  uint64_t heap_data = hh.u64();
  if (!hh.ok || base_ + heap_data + heap_size > bytes_.size()) { *err = path + ": bad local heap"; return false; }
  auto heap_name = [&](uint64_t off) -> std::string {
    if (off >= heap_size) return std::string();
    const char* s = reinterpret_cast<const char*>(bytes_.data() + base_ + heap_data + off);
    size_t maxlen = heap_size - off;
    return std::string(s, strnlen(s, maxlen));
  };

  std::vector<std::pair<std::string, uint64_t>> entries;
  std::set<uint64_t> visited;
  std::function<bool(uint64_t, int)> walk_tree = [&](uint64_t addr, int depth) -> bool {
    if (depth > 32 || visited.count(addr)) return false;
    visited.insert(addr);
    Cursor t{&bytes_, base_ + addr};
    char s[4];
    for (int i = 0; i < 4; i++) s[i] = (char)t.u8();
    if (!t.ok || std::memcmp(s, "TREE", 4) != 0) return false;
    int type = t.u8(), level = t.u8(), used = t.u16();
    t.u64(); t.u64();
    if (type != 0) return false;
    t.u64();  // key 0
    for (int i = 0; i < used; i++) {
      uint64_t child = t.u64();
      t.u64();
      if (!t.ok) return false;
      if (level > 0) {
        if (!walk_tree(child, depth + 1)) return false;
      } else {
        Cursor sn{&bytes_, base_ + child};
        char q[4];
        for (int k = 0; k < 4; k++) q[k] = (char)sn.u8();
        if (!sn.ok || std::memcmp(q, "SNOD", 4) != 0) return false;
        sn.u8(); sn.u8();
        int nsym = sn.u16();
        for (int k = 0; k < nsym; k++) {
          uint64_t noff = sn.u64(), oh = sn.u64();
          sn.u32(); sn.u32(); sn.u64(); sn.u64();
          if (!sn.ok) return false;
          entries.push_back({heap_name(noff), oh});
        }
      }
    }
    return true;
  };
  if (!walk_tree(btree, 0)) { *err = path + ": corrupt group B-tree"; return false; }

  for (auto& e : entries) {
    DatasetInfo d;
    d.name = e.first;
    bool has_layout = false, bad = false;
    bool ok = walk_header(e.second, [&](uint16_t type, Cursor& m, uint64_t msize) {
      if (type == 0x0001) {
        int ver = m.u8();
        d.rank = m.u8();
        int flags = m.u8();
        if (ver == 1) { m.u8(); m.u32(); } else { m.u8(); }
        if (d.rank > 4) { bad = true; return; }
        for (int i = 0; i < d.rank; i++) d.dims[i] = m.u64();
        (void)flags;
      } else if (type == 0x0003) {
        uint8_t b0 = m.u8();
        uint8_t bf0 = m.u8();
        m.u8(); m.u8();
        d.type_class = b0 & 0x0f;
        d.type_size = (int)m.u32();
        if (d.type_class == 0) d.type_signed = (bf0 & 0x08) != 0;
        if ((d.type_class == 0 || d.type_class == 1) && (bf0 & 0x01)) bad = true;  // big endian
      } else if (type == 0x0008) {
        int ver = m.u8();
        if (ver == 1 || ver == 2) {
          int nd = m.u8();
          int cls = m.u8();
          m.u8(); m.u8(); m.u8(); m.u8(); m.u8();
          if (cls == 1) { d.data_addr = m.u64(); for (int i = 0; i < nd; i++) m.u32(); has_layout = true; }
          else if (cls == 0) {
            for (int i = 0; i < nd; i++) m.u32();
            uint32_t cs = m.u32();
            if (m.need(cs)) { d.compact.assign(bytes_.begin() + m.p, bytes_.begin() + m.p + cs); d.is_compact = true; has_layout = true; }
          } else bad = true;
        } else if (ver == 3 || ver == 4) {
          int cls = m.u8();
          if (cls == 1) { d.data_addr = m.u64(); d.data_size = m.u64(); has_layout = true; }
          else if (cls == 0) {
            uint16_t cs = m.u16();
            if (m.need(cs)) { d.compact.assign(bytes_.begin() + m.p, bytes_.begin() + m.p + cs); d.is_compact = true; has_layout = true; }
          } else bad = true;
        } else bad = true;
      }
      (void)msize;
    });
    if (!ok || !has_layout || d.type_class < 0) continue;  // not a dataset this reader understands
    if (bad) { d.type_class = -2; }
    if (d.data_size == 0 && !d.is_compact) d.data_size = d.nelems() * (uint64_t)d.type_size;
    sets_.push_back(d);
  }
  return true;
}

const DatasetInfo* File::find(const std::string& name) const {
  for (auto& d : sets_) if (d.name == name) return &d;
  return nullptr;
}

bool File::read_raw(const DatasetInfo& d, std::vector<uint8_t>* buf, std::string* err) const {
  uint64_t need = d.nelems() * (uint64_t)d.type_size;
  if (d.type_class == -2) { *err = d.name + ": unsupported layout or byte order"; return false; }
  if (d.is_compact) {
    if (d.compact.size() < need) { *err = d.name + ": short compact data"; return false; }
    buf->assign(d.compact.begin(), d.compact.begin() + need);
    return true;
  }
  if (d.data_addr == kUndef) { buf->assign(need, 0); return true; }
  if (base_ + d.data_addr > bytes_.size() || bytes_.size() - (base_ + d.data_addr) < need) {
    *err = d.name + ": data extends past end of file";
    return false;
  }
  buf->assign(bytes_.begin() + base_ + d.data_addr, bytes_.begin() + base_ + d.data_addr + need);
  return true;
}

bool File::read_f64(const std::string& name, double* out, uint64_t n, std::string* err) const {
  const DatasetInfo* d = find(name);
  if (!d) { *err = "dataset '" + name + "' not found"; return false; }
  if (d->nelems() != n) { *err = "dataset '" + name + "' has " + std::to_string(d->nelems()) + " elements, expected " + std::to_string(n); return false; }
  if (d->type_class != 1 || (d->type_size != 8 && d->type_size != 4)) { *err = "dataset '" + name + "' is not floating point"; return false; }
  std::vector<uint8_t> b;
  if (!read_raw(*d, &b, err)) return false;
  if (d->type_size == 8) std::memcpy(out, b.data(), n * 8);
  else for (uint64_t i = 0; i < n; i++) { float v; std::memcpy(&v, b.data() + 4 * i, 4); out[i] = v; }
  return true;
}

bool File::read_i32(const std::string& name, int32_t* out, uint64_t n, std::string* err) const {
  const DatasetInfo* d = find(name);
  if (!d) { *err = "dataset '" + name + "' not found"; return false; }
  if (d->nelems() != n) { *err = "dataset '" + name + "' has " + std::to_string(d->nelems()) + " elements, expected " + std::to_string(n); return false; }
  if (d->type_class != 0 || (d->type_size != 4 && d->type_size != 8)) { *err = "dataset '" + name + "' is not an integer dataset"; return false; }
  std::vector<uint8_t> b;
  if (!read_raw(*d, &b, err)) return false;
  if (d->type_size == 4) { std::memcpy(out, b.data(), n * 4); return true; }
  for (uint64_t i = 0; i < n; i++) {
    int64_t v;
    std::memcpy(&v, b.data() + 8 * i, 8);
    if (v < INT32_MIN || v > INT32_MAX) { *err = "dataset '" + name + "' value out of int32 range"; return false; }
    out[i] = (int32_t)v;
  }
  return true;
}

}  // namespace h5lite
