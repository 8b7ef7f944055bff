// HDF5 output and restart files without an HDF5 library: the structures
// of the published file format that libhdf5's default settings produce.
// All integers little-endian; offsets and lengths 8 bytes.
#include "h5file.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>

namespace edyn {
namespace {

constexpr uint64_t UNDEF = ~0ull;
constexpr int LEAF_K = 4;       // symbol-table node: up to 2 LEAF_K entries
constexpr int INTERNAL_K = 16;  // B-tree node: up to 2 INTERNAL_K children
constexpr size_t SUPERBLOCK_BYTES = 96;
constexpr size_t SNOD_BYTES = 8 + 2 * LEAF_K * 40;
constexpr size_t BTREE_BYTES = 24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8;
constexpr uint16_t MSG_NIL = 0x0, MSG_DATASPACE = 0x1, MSG_DATATYPE = 0x3, MSG_FILL = 0x5, MSG_LAYOUT = 0x8,
                   MSG_ATTR = 0xC, MSG_CONT = 0x10, MSG_STAB = 0x11;
constexpr uint64_t HEAP_FREE_NONE = 1;  // the local heap's end-of-free-list offset

struct Buf {
  std::vector<uint8_t> b;
  void u8(unsigned v) { b.push_back((uint8_t)v); }
  void u16(unsigned v) { for (int i = 0; i < 2; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
  void u32(uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
  void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
  void raw(const void* p, size_t n) { b.insert(b.end(), (const uint8_t*)p, (const uint8_t*)p + n); }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void pad8() { while (b.size() % 8) b.push_back(0); }
};

size_t align8(size_t n) { return (n + 7) & ~(size_t)7; }

// IEEE float64, little-endian (H5T_IEEE_F64LE = H5T_NATIVE_DOUBLE here)
std::vector<uint8_t> dtype_f64() {
  Buf d;
  d.u8(0x11);  // version 1, class 1 (floating point)
  d.u8(0x20);  // little-endian, mantissa normalisation "implied msb"
  d.u8(63);    // sign bit
  d.u8(0);
  d.u32(8);
  d.u16(0);    // bit offset
  d.u16(64);   // precision
  d.u8(52);    // exponent location
  d.u8(11);    // exponent size
  d.u8(0);     // mantissa location
  d.u8(52);    // mantissa size
  d.u32(1023); // exponent bias
  return d.b;
}

// signed int32, little-endian (H5T_NATIVE_INTEGER of the Fortran API)
std::vector<uint8_t> dtype_i32() {
  Buf d;
  d.u8(0x10);  // version 1, class 0 (fixed point)
  d.u8(0x08);  // little-endian, signed
  d.u8(0);
  d.u8(0);
  d.u32(4);
  d.u16(0);
  d.u16(32);
  return d.b;
}

// simple rank-1 dataspace of n elements, no maximum dimensions
std::vector<uint8_t> dspace_1d(uint64_t n) {
  Buf d;
  d.u8(1);  // version 1
  d.u8(1);  // rank
  d.u8(0);  // flags
  d.u8(0);
  d.u32(0);
  d.u64(n);
  return d.b;
}

struct Message {
  uint16_t type;
  uint8_t flags;
  std::vector<uint8_t> data;
};

// version-1 object header: prefix, then each message with its data padded
// to eight bytes
std::vector<uint8_t> object_header(const std::vector<Message>& msgs) {
  size_t chunk = 0;
  for (const Message& m : msgs) chunk += 8 + align8(m.data.size());
  Buf h;
  h.u8(1);
  h.u8(0);
  h.u16((unsigned)msgs.size());
  h.u32(1);  // reference count
  h.u32((uint32_t)chunk);
  h.u32(0);  // alignment of the messages
  for (const Message& m : msgs) {
    h.u16(m.type);
    h.u16((unsigned)align8(m.data.size()));
    h.u8(m.flags);
    h.zeros(3);
    h.raw(m.data.data(), m.data.size());
    h.pad8();
  }
  return h.b;
}

Message attribute(const H5Attr& a) {
  const std::vector<uint8_t> dt = a.is_int ? dtype_i32() : dtype_f64();
  const std::vector<uint8_t> ds = dspace_1d(1);
  Buf m;
  m.u8(1);  // version 1: name, datatype and dataspace each padded to 8
  m.u8(0);
  m.u16((unsigned)(a.name.size() + 1));
  m.u16((unsigned)dt.size());
  m.u16((unsigned)ds.size());
  m.raw(a.name.data(), a.name.size());
  m.u8(0);
  m.pad8();
  m.raw(dt.data(), dt.size());
  m.pad8();
  m.raw(ds.data(), ds.size());
  m.pad8();
  if (a.is_int) {
    m.u32((uint32_t)(int32_t)a.value);
  } else {
    uint64_t bits;
    std::memcpy(&bits, &a.value, 8);
    m.u64(bits);
  }
  return {MSG_ATTR, 0, m.b};
}

uint16_t rd16(const uint8_t* p) { return (uint16_t)(p[0] | (p[1] << 8)); }
uint32_t rd32(const uint8_t* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24); }
uint64_t rd64(const uint8_t* p) { return (uint64_t)rd32(p) | ((uint64_t)rd32(p + 4) << 32); }
uint64_t rdn(const uint8_t* p, int n, bool be) {
  uint64_t v = 0;
  for (int i = 0; i < n; ++i) v |= (uint64_t)p[be ? n - 1 - i : i] << (8 * i);
  return v;
}

}  // namespace

// Fortran's Ew.d with w = 11, d = 5: 0.ddddd and a signed two-digit exponent
// (three digits without the E beyond +-99), the digits rounded to nearest.
std::string step_group_name(int nout, double x) {
  char out[96];
  if (x == 0.0) {
    std::snprintf(out, sizeof(out), "nout%06d_time0.00000E+00", nout);
    return out;
  }
  char b[64];
  std::snprintf(b, sizeof(b), "%.4E", std::fabs(x));  // d.ddddE+xx
  const int e = std::atoi(std::strchr(b, 'E') + 1) + 1;
  const std::string dig = std::string(1, b[0]) + std::string(b + 2, 4);
  const char* sg = x < 0 ? "-" : "";
  if (e >= -99 && e <= 99)
    std::snprintf(out, sizeof(out), "nout%06d_time%s0.%sE%c%02d", nout, sg, dig.c_str(), e < 0 ? '-' : '+', std::abs(e));
  else
    std::snprintf(out, sizeof(out), "nout%06d_time%s0.%s%c%03d", nout, sg, dig.c_str(), e < 0 ? '-' : '+', std::abs(e));
  return out;
}

// ---------------------------------------------------------------------------
// Writer
// ---------------------------------------------------------------------------
H5Writer::~H5Writer() {
  std::string err;
  close(err);
}

uint64_t H5Writer::append(const std::vector<uint8_t>& bytes) {
  const uint64_t at = eof_;
  if (std::fseek(f_, (long)at, SEEK_SET) != 0 || std::fwrite(bytes.data(), 1, bytes.size(), f_) != bytes.size())
    ok_ = false;
  eof_ += bytes.size();
  return at;
}

// A group's index: its local heap of member names, the symbol-table nodes
// holding the members in name order, and one leaf B-tree node over them.
bool H5Writer::write_symbol_table(std::vector<Entry> entries, uint64_t& btree, uint64_t& heap, std::string& err) {
  std::sort(entries.begin(), entries.end(), [](const Entry& a, const Entry& b) { return a.name < b.name; });
  for (size_t i = 1; i < entries.size(); ++i)
    if (entries[i].name == entries[i - 1].name) {
      err = "duplicate member name '" + entries[i].name + "'";
      return false;
    }
  const size_t per_node = 2 * LEAF_K;
  const size_t nodes = (entries.size() + per_node - 1) / per_node;
  if (nodes > 2 * INTERNAL_K) {
    err = "more than " + std::to_string(2 * INTERNAL_K * per_node) + " members in one group";
    return false;
  }
  // heap data: the empty name at offset 0, then every name, each padded to 8
  Buf data;
  data.zeros(8);
  std::vector<uint64_t> name_off(entries.size());
  for (size_t i = 0; i < entries.size(); ++i) {
    name_off[i] = data.b.size();
    data.raw(entries[i].name.data(), entries[i].name.size());
    data.u8(0);
    data.pad8();
  }
  Buf h;
  h.raw("HEAP", 4);
  h.u8(0);
  h.zeros(3);
  h.u64(data.b.size());
  h.u64(HEAP_FREE_NONE);
  const uint64_t heap_at = eof_;
  h.u64(heap_at + 32);  // the data segment follows the header
  h.raw(data.b.data(), data.b.size());
  heap = append(h.b);
  // symbol-table nodes
  std::vector<uint64_t> node_at(nodes);
  for (size_t nd = 0; nd < nodes; ++nd) {
    const size_t i0 = nd * per_node, i1 = std::min(entries.size(), i0 + per_node);
    Buf s;
    s.raw("SNOD", 4);
    s.u8(1);
    s.u8(0);
    s.u16((unsigned)(i1 - i0));
    for (size_t i = i0; i < i1; ++i) {
      s.u64(name_off[i]);
      s.u64(entries[i].ohdr);
      s.u32(entries[i].group ? 1 : 0);  // groups cache their symbol table's addresses
      s.u32(0);
      s.u64(entries[i].group ? entries[i].btree : 0);
      s.u64(entries[i].group ? entries[i].heap : 0);
    }
    s.b.resize(SNOD_BYTES, 0);
    node_at[nd] = append(s.b);
  }
  // B-tree leaf: key 0 is the empty name, key i+1 the last name of child i
  Buf t;
  t.raw("TREE", 4);
  t.u8(0);  // group node
  t.u8(0);  // leaf
  t.u16((unsigned)nodes);
  t.u64(UNDEF);
  t.u64(UNDEF);
  t.u64(0);
  for (size_t nd = 0; nd < nodes; ++nd) {
    const size_t last = std::min(entries.size(), (nd + 1) * per_node) - 1;
    t.u64(node_at[nd]);
    t.u64(name_off[last]);
  }
  t.b.resize(BTREE_BYTES, 0);
  btree = append(t.b);
  if (!ok_) err = "write failed";
  return ok_;
}

bool H5Writer::rewrite_superblock(std::string& err) {
  Buf s;
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  s.raw(sig, 8);
  s.u8(0);  // superblock version
  s.u8(0);  // free-space storage version
  s.u8(0);  // root group symbol table entry version
  s.u8(0);
  s.u8(0);  // shared header message format version
  s.u8(8);  // size of offsets
  s.u8(8);  // size of lengths
  s.u8(0);
  s.u16(LEAF_K);
  s.u16(INTERNAL_K);
  s.u32(0);  // file consistency flags
  s.u64(0);  // base address
  s.u64(UNDEF);  // free-space info
  s.u64(eof_);
  s.u64(UNDEF);  // driver information block
  // root group symbol table entry
  s.u64(0);
  s.u64(root_ohdr_);
  s.u32(1);
  s.u32(0);
  s.u64(root_btree_);
  s.u64(root_heap_);
  if (s.b.size() != SUPERBLOCK_BYTES) {
    err = "superblock size";
    return false;
  }
  if (std::fseek(f_, 0, SEEK_SET) != 0 || std::fwrite(s.b.data(), 1, s.b.size(), f_) != s.b.size() ||
      std::fflush(f_) != 0) {
    err = "superblock write failed";
    return false;
  }
  return true;
}

bool H5Writer::create(const std::string& path, std::string& err) {
  close(err);
  err.clear();
  f_ = std::fopen(path.c_str(), "w+b");
  if (!f_) {
    err = "cannot create " + path;
    return false;
  }
  path_ = path;
  ok_ = true;
  root_.clear();
  eof_ = 0;
  append(std::vector<uint8_t>(SUPERBLOCK_BYTES, 0));
  if (!write_symbol_table({}, root_btree_, root_heap_, err)) return false;
  std::vector<uint8_t> stab;
  {
    Buf m;
    m.u64(root_btree_);
    m.u64(root_heap_);
    stab = m.b;
  }
  root_ohdr_ = append(object_header({{MSG_STAB, 1, stab}}));
  return rewrite_superblock(err);
}

bool H5Writer::add_group(const std::string& name, const std::vector<H5Attr>& attrs,
                         const std::vector<std::string>& row_names, const double* rows, int64_t n, std::string& err) {
  if (!f_) {
    err = "no file is open";
    return false;
  }
  if (n < 0 || (n > 0 && !rows)) {
    err = "bad rows";
    return false;
  }
  for (const Entry& e : root_)
    if (e.name == name) {
      err = "group '" + name + "' exists";
      return false;
    }
  std::vector<Entry> members;
  const uint64_t bytes = (uint64_t)n * 8;
  for (size_t r = 0; r < row_names.size(); ++r) {
    // raw data (little-endian float64 rows, as in memory on both hosts)
    const uint64_t at = eof_;
    if (bytes) {
      if (std::fseek(f_, (long)at, SEEK_SET) != 0 ||
          std::fwrite(rows + (size_t)r * (size_t)n, 8, (size_t)n, f_) != (size_t)n)
        ok_ = false;
      eof_ += bytes;
    }
    Buf fill;
    fill.u8(1);  // version 1: allocation late, write if set, defined, no value (size 0)
    fill.u8(2);
    fill.u8(2);
    fill.u8(1);
    fill.u32(0);
    Buf lay;
    lay.u8(3);  // version 3
    lay.u8(1);  // contiguous
    lay.u64(bytes ? at : UNDEF);
    lay.u64(bytes);
    Entry e;
    e.name = row_names[r];
    e.ohdr = append(object_header({{MSG_DATASPACE, 0, dspace_1d((uint64_t)n)},
                                   {MSG_DATATYPE, 1, dtype_f64()},
                                   {MSG_FILL, 1, fill.b},
                                   {MSG_LAYOUT, 0, lay.b}}));
    members.push_back(e);
  }
  Entry g;
  g.name = name;
  g.group = true;
  if (!write_symbol_table(members, g.btree, g.heap, err)) return false;
  std::vector<Message> msgs;
  {
    Buf m;
    m.u64(g.btree);
    m.u64(g.heap);
    msgs.push_back({MSG_STAB, 1, m.b});
  }
  for (const H5Attr& a : attrs) msgs.push_back(attribute(a));
  g.ohdr = append(object_header(msgs));
  root_.push_back(g);
  if (!write_symbol_table(root_, root_btree_, root_heap_, err)) return false;
  {
    Buf m;
    m.u64(root_btree_);
    m.u64(root_heap_);
    root_ohdr_ = append(object_header({{MSG_STAB, 1, m.b}}));
  }
  if (!ok_) {
    err = "write failed";
    return false;
  }
  return rewrite_superblock(err);
}

bool H5Writer::close(std::string& err) {
  if (!f_) return true;
  const bool ok = ok_ && std::fflush(f_) == 0;
  const bool closed = std::fclose(f_) == 0;
  f_ = nullptr;
  if (!ok || !closed) {
    err = "close failed";
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Reader
// ---------------------------------------------------------------------------
H5Reader::~H5Reader() {
  if (fp_) std::fclose(fp_);
}

bool H5Reader::read_at(uint64_t addr, size_t len, std::vector<uint8_t>& out, std::string& err) {
  const uint64_t a = base_ + addr;
  if (addr == UNDEF || a < addr || a > size_ || len > size_ - a) {
    err = "address out of the file";
    return false;
  }
  out.resize(len);
  if (len && (std::fseek(fp_, (long)a, SEEK_SET) != 0 || std::fread(out.data(), 1, len, fp_) != len)) {
    err = "read failed";
    return false;
  }
  return true;
}

bool H5Reader::open(const std::string& path, std::string& err) {
  if (fp_) std::fclose(fp_);
  fp_ = std::fopen(path.c_str(), "rb");
  if (!fp_) {
    err = "cannot open " + path;
    return false;
  }
  std::fseek(fp_, 0, SEEK_END);
  size_ = (uint64_t)std::ftell(fp_);
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  // the superblock sits at 0 or at a power of two from 512 on (user block)
  for (uint64_t at = 0; at + 8 <= size_; at = at ? 2 * at : 512) {
    base_ = 0;
    std::vector<uint8_t> b;
    if (!read_at(at, std::min<uint64_t>(size_ - at, 128), b, err)) return false;
    if (b.size() < 8 || std::memcmp(b.data(), sig, 8) != 0) continue;
    const int ver = b[8];
    if (ver > 1) {
      err = "superblock version " + std::to_string(ver) + " (only 0 and 1)";
      return false;
    }
    if (b[13] != 8 || b[14] != 8) {
      err = "offsets and lengths other than 8 bytes";
      return false;
    }
    leaf_k_ = rd16(&b[16]);
    internal_k_ = rd16(&b[18]);
    size_t p = 24 + (ver == 1 ? 4 : 0);
    if (b.size() < p + 32 + 40) {
      err = "truncated superblock";
      return false;
    }
    base_ = rd64(&b[p]);
    root_ohdr_ = rd64(&b[p + 32 + 8]);
    return true;
  }
  err = "no HDF5 superblock";
  return false;
}

bool H5Reader::header(uint64_t addr, std::vector<Msg>& msgs, std::string& err) {
  std::vector<uint8_t> pre;
  if (!read_at(addr, 16, pre, err)) return false;
  if (pre[0] != 1) {
    err = "object header version " + std::to_string(pre[0]) + " (only 1)";
    return false;
  }
  const unsigned nmsgs = rd16(&pre[2]);
  std::vector<std::pair<uint64_t, uint64_t>> chunks{{addr + 16, rd32(&pre[8])}};
  unsigned seen = 0;
  for (size_t c = 0; c < chunks.size() && c < 4096; ++c) {
    std::vector<uint8_t> b;
    if (!read_at(chunks[c].first, (size_t)chunks[c].second, b, err)) return false;
    size_t p = 0;
    while (p + 8 <= b.size() && seen < nmsgs) {
      const uint16_t type = rd16(&b[p]);
      const uint16_t sz = rd16(&b[p + 2]);
      const uint8_t flags = b[p + 4];
      if (p + 8 + sz > b.size()) {
        err = "message runs past its header chunk";
        return false;
      }
      ++seen;
      if (type == MSG_CONT) {
        if (sz < 16) {
          err = "short continuation message";
          return false;
        }
        chunks.push_back({rd64(&b[p + 8]), rd64(&b[p + 16])});
      } else if (type != MSG_NIL) {
        if (flags & 0x02) {
          err = "shared object header messages are not supported";
          return false;
        }
        msgs.push_back({type, flags, std::vector<uint8_t>(b.begin() + p + 8, b.begin() + p + 8 + sz)});
      }
      p += 8 + sz;
    }
  }
  return true;
}

bool H5Reader::btree_walk(uint64_t addr, const std::vector<uint8_t>& heap, std::vector<H5Object>& out, int depth,
                          std::string& err) {
  if (depth > 32) {
    err = "B-tree too deep";
    return false;
  }
  std::vector<uint8_t> h;
  if (!read_at(addr, 24, h, err)) return false;
  if (std::memcmp(h.data(), "TREE", 4) != 0 || h[4] != 0) {
    err = "not a group B-tree node";
    return false;
  }
  const int level = h[5];
  const unsigned used = rd16(&h[6]);
  std::vector<uint8_t> kc;
  if (!read_at(addr + 24, (size_t)(2 * used + 1) * 8, kc, err)) return false;
  for (unsigned i = 0; i < used; ++i) {
    const uint64_t child = rd64(&kc[8 + 16 * i]);
    if (level > 0) {
      if (!btree_walk(child, heap, out, depth + 1, err)) return false;
      continue;
    }
    std::vector<uint8_t> s;
    if (!read_at(child, 8, s, err)) return false;
    if (std::memcmp(s.data(), "SNOD", 4) != 0) {
      err = "not a symbol-table node";
      return false;
    }
    const unsigned nsym = rd16(&s[6]);
    std::vector<uint8_t> ent;
    if (!read_at(child + 8, (size_t)nsym * 40, ent, err)) return false;
    for (unsigned j = 0; j < nsym; ++j) {
      const uint8_t* e = &ent[40 * j];
      const uint64_t off = rd64(e);
      if (off >= heap.size()) {
        err = "name offset outside the local heap";
        return false;
      }
      const char* nm = (const char*)&heap[off];
      const size_t len = strnlen(nm, heap.size() - off);
      H5Object o;
      o.name.assign(nm, len);
      o.ohdr = rd64(e + 8);
      out.push_back(o);
    }
  }
  return true;
}

bool H5Reader::group_members(uint64_t ohdr, std::vector<H5Object>& out, std::string& err) {
  std::vector<Msg> msgs;
  if (!header(ohdr, msgs, err)) return false;
  const Msg* st = nullptr;
  for (const Msg& m : msgs)
    if (m.type == MSG_STAB) st = &m;
  if (!st || st->data.size() < 16) {
    err = "not a symbol-table group";
    return false;
  }
  const uint64_t bt = rd64(&st->data[0]), hp = rd64(&st->data[8]);
  std::vector<uint8_t> hh;
  if (!read_at(hp, 32, hh, err)) return false;
  if (std::memcmp(hh.data(), "HEAP", 4) != 0) {
    err = "not a local heap";
    return false;
  }
  std::vector<uint8_t> heap;
  if (!read_at(rd64(&hh[24]), (size_t)rd64(&hh[8]), heap, err)) return false;
  out.clear();
  if (!btree_walk(bt, heap, out, 0, err)) return false;
  for (H5Object& o : out) {
    std::vector<Msg> m;
    if (!header(o.ohdr, m, err)) return false;
    for (const Msg& x : m)
      if (x.type == MSG_STAB) o.group = true;
  }
  return true;
}

bool H5Reader::resolve(const std::string& path, uint64_t& ohdr, std::string& err) {
  ohdr = root_ohdr_;
  size_t p = 0;
  while (p < path.size()) {
    size_t q = path.find('/', p);
    if (q == std::string::npos) q = path.size();
    const std::string part = path.substr(p, q - p);
    p = q + 1;
    if (part.empty() || part == ".") continue;
    std::vector<H5Object> mem;
    if (!group_members(ohdr, mem, err)) return false;
    bool found = false;
    for (const H5Object& o : mem)
      if (o.name == part) {
        ohdr = o.ohdr;
        found = true;
        break;
      }
    if (!found) {
      err = "no member '" + part + "'";
      return false;
    }
  }
  return true;
}

bool H5Reader::list(const std::string& group, std::vector<H5Object>& out, std::string& err) {
  uint64_t oh;
  if (!resolve(group, oh, err)) return false;
  return group_members(oh, out, err);
}

namespace {
bool parse_dspace(const std::vector<uint8_t>& d, std::vector<uint64_t>& dims, std::string& err) {
  dims.clear();
  if (d.size() < 4) {
    err = "short dataspace";
    return false;
  }
  const int ver = d[0], rank = d[1];
  size_t p;
  if (ver == 1) {
    p = 8;
  } else if (ver == 2) {
    p = 4;
    if (d[3] == 2) return true;  // null dataspace: no elements
  } else {
    err = "dataspace version " + std::to_string(ver);
    return false;
  }
  if (d.size() < p + 8 * (size_t)rank) {
    err = "short dataspace";
    return false;
  }
  for (int i = 0; i < rank; ++i) dims.push_back(rd64(&d[p + 8 * i]));
  return true;
}

// element decoder of a datatype message: float, integer or string
struct DType {
  int cls = -1;
  size_t size = 0;
  bool be = false, sgn = false;
};

bool parse_dtype(const std::vector<uint8_t>& d, DType& t, std::string& err) {
  if (d.size() < 8) {
    err = "short datatype";
    return false;
  }
  t.cls = d[0] & 0x0f;
  t.size = rd32(&d[4]);
  t.be = (d[1] & 0x01) != 0;
  t.sgn = (d[1] & 0x08) != 0;
  if (t.cls == 1 && (t.size == 4 || t.size == 8)) return true;
  if (t.cls == 0 && (t.size == 1 || t.size == 2 || t.size == 4 || t.size == 8)) return true;
  if (t.cls == 3) return true;
  err = "datatype class " + std::to_string(t.cls) + " of " + std::to_string(t.size) + " bytes is not supported";
  return false;
}

bool decode(const DType& t, const uint8_t* p, size_t count, H5Value& v) {
  if (t.cls == 3) {
    v.is_string = true;
    v.text.assign((const char*)p, strnlen((const char*)p, t.size * count));
    return true;
  }
  v.data.resize(count);
  for (size_t i = 0; i < count; ++i) {
    const uint64_t raw = rdn(p + i * t.size, (int)t.size, t.be);
    if (t.cls == 1) {
      if (t.size == 8) {
        double x;
        std::memcpy(&x, &raw, 8);
        v.data[i] = x;
      } else {
        const uint32_t r32 = (uint32_t)raw;
        float x;
        std::memcpy(&x, &r32, 4);
        v.data[i] = x;
      }
    } else if (t.sgn) {
      const int sh = 64 - 8 * (int)t.size;
      v.data[i] = (double)((int64_t)(raw << sh) >> sh);
    } else {
      v.data[i] = (double)raw;
    }
  }
  return true;
}
}  // namespace

bool H5Reader::read_dataset(const std::string& path, H5Value& v, std::string& err) {
  uint64_t oh;
  if (!resolve(path, oh, err)) return false;
  std::vector<Msg> msgs;
  if (!header(oh, msgs, err)) return false;
  const Msg *ds = nullptr, *dt = nullptr, *ly = nullptr;
  for (const Msg& m : msgs) {
    if (m.type == MSG_DATASPACE) ds = &m;
    if (m.type == MSG_DATATYPE) dt = &m;
    if (m.type == MSG_LAYOUT) ly = &m;
  }
  if (!ds || !dt || !ly) {
    err = "'" + path + "' is not a dataset";
    return false;
  }
  DType t;
  if (!parse_dspace(ds->data, v.dims, err) || !parse_dtype(dt->data, t, err)) return false;
  size_t count = 1;
  for (uint64_t d : v.dims) count *= (size_t)d;
  const size_t bytes = count * t.size;
  const std::vector<uint8_t>& L = ly->data;
  std::vector<uint8_t> raw;
  if (L.size() < 2) {
    err = "short layout";
    return false;
  }
  if (L[0] == 3) {
    if (L[1] == 1) {  // contiguous
      const uint64_t addr = rd64(&L[2]);
      if (addr == UNDEF) {
        raw.assign(bytes, 0);
      } else if (!read_at(addr, bytes, raw, err)) {
        return false;
      }
    } else if (L[1] == 0) {  // compact
      const size_t sz = rd16(&L[2]);
      if (sz < bytes || L.size() < 4 + bytes) {
        err = "short compact data";
        return false;
      }
      raw.assign(L.begin() + 4, L.begin() + 4 + bytes);
    } else {
      err = "chunked datasets are not supported";
      return false;
    }
  } else if (L[0] == 1 || L[0] == 2) {
    const int dimsz = L[1];
    const int cls = L[2];
    if (cls == 1) {
      const uint64_t addr = rd64(&L[8]);
      if (addr == UNDEF) {
        raw.assign(bytes, 0);
      } else if (!read_at(addr, bytes, raw, err)) {
        return false;
      }
    } else if (cls == 0) {
      const size_t p = 8 + 4 * (size_t)dimsz;
      if (L.size() < p + 4 + bytes) {
        err = "short compact data";
        return false;
      }
      raw.assign(L.begin() + p + 4, L.begin() + p + 4 + bytes);
    } else {
      err = "chunked datasets are not supported";
      return false;
    }
  } else {
    err = "layout version " + std::to_string(L[0]);
    return false;
  }
  return decode(t, raw.data(), count, v);
}

namespace {
struct AttrView {
  std::string name;
  std::vector<uint8_t> dt, ds;
  const uint8_t* data = nullptr;
  size_t data_len = 0;
};

bool parse_attr(const std::vector<uint8_t>& m, AttrView& a, std::string& err) {
  if (m.size() < 8) {
    err = "short attribute";
    return false;
  }
  const int ver = m[0];
  const size_t nl = rd16(&m[2]), tl = rd16(&m[4]), sl = rd16(&m[6]);
  size_t p = ver == 3 ? 9 : 8;
  auto adv = [&](size_t n) { return ver == 1 ? align8(n) : n; };
  if (ver < 1 || ver > 3 || m.size() < p + adv(nl) + adv(tl) + adv(sl)) {
    err = "bad attribute message";
    return false;
  }
  a.name.assign((const char*)&m[p], strnlen((const char*)&m[p], nl));
  p += adv(nl);
  a.dt.assign(m.begin() + p, m.begin() + p + tl);
  p += adv(tl);
  a.ds.assign(m.begin() + p, m.begin() + p + sl);
  p += adv(sl);
  a.data = m.data() + p;
  a.data_len = m.size() - p;
  return true;
}
}  // namespace

bool H5Reader::attr_names(const std::string& object, std::vector<std::string>& out, std::string& err) {
  uint64_t oh;
  if (!resolve(object, oh, err)) return false;
  std::vector<Msg> msgs;
  if (!header(oh, msgs, err)) return false;
  out.clear();
  for (const Msg& m : msgs)
    if (m.type == MSG_ATTR) {
      AttrView a;
      if (!parse_attr(m.data, a, err)) return false;
      out.push_back(a.name);
    }
  return true;
}

bool H5Reader::read_attr(const std::string& object, const std::string& name, H5Value& v, std::string& err) {
  uint64_t oh;
  if (!resolve(object, oh, err)) return false;
  std::vector<Msg> msgs;
  if (!header(oh, msgs, err)) return false;
  for (const Msg& m : msgs) {
    if (m.type != MSG_ATTR) continue;
    AttrView a;
    if (!parse_attr(m.data, a, err)) return false;
    if (a.name != name) continue;
    DType t;
    if (!parse_dtype(a.dt, t, err)) return false;
    if (a.ds.size() >= 2 && a.ds[1] == 0) {
      v.dims.clear();  // scalar
    } else if (!parse_dspace(a.ds, v.dims, err)) {
      return false;
    }
    size_t count = 1;
    for (uint64_t d : v.dims) count *= (size_t)d;
    if (count * t.size > a.data_len) {
      err = "short attribute data";
      return false;
    }
    return decode(t, a.data, count, v);
  }
  err = "no attribute '" + name + "'";
  return false;
}

}  // namespace edyn

// ---------------------------------------------------------------------------
// C ABI of include/edyn_h5.h
// ---------------------------------------------------------------------------
#include "../../include/edyn_gpu.h"
#include "../../include/edyn_h5.h"

namespace {
thread_local std::string g_h5_err;

int h5_fail(int code, const std::string& msg) {
  g_h5_err = msg;
  return code;
}

int copy_text(const std::string& s, char* buf, long long len) {
  if (!buf || len <= 0) return h5_fail(EDYN_E_ARG, "no buffer");
  if ((long long)s.size() + 1 > len) return h5_fail(EDYN_E_ARG, "buffer of " + std::to_string(len) + " bytes too small");
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return EDYN_OK;
}
}  // namespace

extern "C" {

int edyn_h5_create(const char* path, void** h) {
  if (!path || !h) return h5_fail(EDYN_E_ARG, "null argument");
  *h = nullptr;
  auto* w = new (std::nothrow) edyn::H5Writer;
  if (!w) return h5_fail(EDYN_E_ARG, "out of memory");
  std::string err;
  if (!w->create(path, err)) {
    delete w;
    return h5_fail(EDYN_E_IO, err);
  }
  *h = w;
  return EDYN_OK;
}

int edyn_h5_add_group(void* h, const char* name, int nattr, const char* const* attr_names, const int* attr_is_int,
                      const double* attr_values, int nrow, const char* const* row_names, const double* rows,
                      long long n) {
  if (!h || !name || nattr < 0 || nrow < 0 || n < 0 || (nattr && (!attr_names || !attr_is_int || !attr_values)) ||
      (nrow && !row_names) || (nrow && n && !rows))
    return h5_fail(EDYN_E_ARG, "bad arguments");
  std::vector<edyn::H5Attr> attrs;
  for (int a = 0; a < nattr; ++a) {
    if (!attr_names[a]) return h5_fail(EDYN_E_ARG, "null attribute name");
    attrs.push_back({attr_names[a], attr_is_int[a] != 0, attr_values[a]});
  }
  std::vector<std::string> names;
  for (int r = 0; r < nrow; ++r) {
    if (!row_names[r] || !row_names[r][0]) return h5_fail(EDYN_E_ARG, "empty dataset name");
    names.push_back(row_names[r]);
  }
  std::string err;
  if (!static_cast<edyn::H5Writer*>(h)->add_group(name, attrs, names, rows, n, err)) return h5_fail(EDYN_E_IO, err);
  return EDYN_OK;
}

int edyn_h5_close(void* h) {
  if (!h) return EDYN_OK;
  auto* w = static_cast<edyn::H5Writer*>(h);
  std::string err;
  const bool ok = w->close(err);
  delete w;
  return ok ? EDYN_OK : h5_fail(EDYN_E_IO, err);
}

int edyn_h5_list(const char* path, const char* group, char* buf, long long len) {
  if (!path) return h5_fail(EDYN_E_ARG, "null path");
  edyn::H5Reader r;
  std::string err;
  std::vector<edyn::H5Object> m;
  if (!r.open(path, err) || !r.list(group ? group : "", m, err)) return h5_fail(EDYN_E_IO, err);
  std::string s;
  for (const auto& o : m) s += o.name + (o.group ? "/\n" : "\n");
  return copy_text(s, buf, len);
}

int edyn_h5_read(const char* path, const char* dataset, double* out, long long cap, long long* n) {
  if (!path || !dataset) return h5_fail(EDYN_E_ARG, "null argument");
  edyn::H5Reader r;
  std::string err;
  edyn::H5Value v;
  if (!r.open(path, err) || !r.read_dataset(dataset, v, err)) return h5_fail(EDYN_E_IO, err);
  if (v.is_string) return h5_fail(EDYN_E_ARG, "string dataset");
  if (n) *n = (long long)v.data.size();
  if (out) std::memcpy(out, v.data.data(), std::min<size_t>(v.data.size(), (size_t)std::max(cap, 0ll)) * 8);
  return EDYN_OK;
}

int edyn_h5_attr(const char* path, const char* object, const char* name, double* out, long long cap, long long* n,
                 char* buf, long long len) {
  if (!path || !object || !name) return h5_fail(EDYN_E_ARG, "null argument");
  edyn::H5Reader r;
  std::string err;
  edyn::H5Value v;
  if (!r.open(path, err) || !r.read_attr(object, name, v, err)) return h5_fail(EDYN_E_IO, err);
  if (v.is_string) {
    if (n) *n = 0;
    return buf ? copy_text(v.text, buf, len) : EDYN_OK;
  }
  if (n) *n = (long long)v.data.size();
  if (out) std::memcpy(out, v.data.data(), std::min<size_t>(v.data.size(), (size_t)std::max(cap, 0ll)) * 8);
  return EDYN_OK;
}

int edyn_h5_attr_names(const char* path, const char* object, char* buf, long long len) {
  if (!path || !object) return h5_fail(EDYN_E_ARG, "null argument");
  edyn::H5Reader r;
  std::string err;
  std::vector<std::string> names;
  if (!r.open(path, err) || !r.attr_names(object, names, err)) return h5_fail(EDYN_E_IO, err);
  std::string s;
  for (const auto& a : names) s += a + "\n";
  return copy_text(s, buf, len);
}

int edyn_h5_step_name(int nout, double time, char* buf, int len) {
  if (nout < 0 || nout > 999999) return h5_fail(EDYN_E_ARG, "nout out of i6.6");
  return copy_text(edyn::step_group_name(nout, time), buf, len);
}

const char* edyn_h5_error(void) { return g_h5_err.c_str(); }

}  // extern "C"
