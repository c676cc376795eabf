// Minimal HDF5 writer/reader for the reference's result layouts (see
// wlg_h5.h).  Structures follow the public HDF5 File Format Specification
// version 3.0: superblock version 2 (section II.A), version-2 object headers
// (IV.A.1.b), Dataspace (IV.A.2.b, version 2), Datatype (IV.A.2.d: fixed-point,
// floating-point, string, compound version 1), Fill Value (IV.A.2.f, version
// 3), Link Info (IV.A.2.c), Group Info (IV.A.2.k), Link (IV.A.2.g, version 1),
// Data Layout (IV.A.2.i, version 3, contiguous) and Attribute (IV.A.2.m,
// version 3) messages.  All addresses and lengths are 8 bytes, little-endian.

#include "wlg_h5.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>

namespace wlg::h5 {

uint32_t lookup3(const uint8_t* k, size_t length, uint32_t init)
{
  auto rot = [](uint32_t x, int r) { return (x << r) | (x >> (32 - r)); };
  uint32_t a, b, c;
  a = b = c = 0xdeadbeefu + static_cast<uint32_t>(length) + init;
  auto word = [&](const uint8_t* p) {
    return static_cast<uint32_t>(p[0]) | static_cast<uint32_t>(p[1]) << 8 | static_cast<uint32_t>(p[2]) << 16 |
           static_cast<uint32_t>(p[3]) << 24;
  };
  while (length > 12) {
    a += word(k);
    b += word(k + 4);
    c += word(k + 8);
    a -= c; a ^= rot(c, 4);  c += b;
    b -= a; b ^= rot(a, 6);  a += c;
    c -= b; c ^= rot(b, 8);  b += a;
    a -= c; a ^= rot(c, 16); c += b;
    b -= a; b ^= rot(a, 19); a += c;
    c -= b; c ^= rot(b, 4);  b += a;
    length -= 12;
    k += 12;
  }
  if (length == 0) return c;
  uint8_t tail[12] = {};
  std::memcpy(tail, k, length);
  a += word(tail);
  b += word(tail + 4);
  c += word(tail + 8);
  c ^= b; c -= rot(b, 14);
  a ^= c; a -= rot(c, 11);
  b ^= a; b -= rot(a, 25);
  c ^= b; c -= rot(b, 16);
  a ^= c; a -= rot(c, 4);
  b ^= a; b -= rot(a, 14);
  c ^= b; c -= rot(b, 24);
  return c;
}

Group& Group::group(const std::string& name)
{
  auto& g = groups[name];
  if (!g) g = std::make_unique<Group>();
  return *g;
}

Dataset make_u64(const std::vector<uint64_t>& v)
{
  Dataset d;
  d.type = Type::u64;
  d.count = v.size();
  d.bytes.resize(8 * v.size());
  for (size_t i = 0; i < v.size(); ++i)
    for (int j = 0; j < 8; ++j) d.bytes[8 * i + j] = static_cast<uint8_t>(v[i] >> (8 * j));
  return d;
}

Dataset make_i8(const std::vector<int8_t>& v)
{
  Dataset d;
  d.type = Type::i8;
  d.count = v.size();
  d.bytes.assign(reinterpret_cast<const uint8_t*>(v.data()), reinterpret_cast<const uint8_t*>(v.data()) + v.size());
  return d;
}

Dataset make_key_value(const std::vector<std::pair<int32_t, double>>& v)
{
  Dataset d;
  d.type = Type::key_value;
  d.count = v.size();
  d.bytes.assign(16 * v.size(), 0);
  for (size_t i = 0; i < v.size(); ++i) {
    const uint32_t key = static_cast<uint32_t>(v[i].first);
    uint64_t val;
    std::memcpy(&val, &v[i].second, 8);
    for (int j = 0; j < 4; ++j) d.bytes[16 * i + j] = static_cast<uint8_t>(key >> (8 * j));
    for (int j = 0; j < 8; ++j) d.bytes[16 * i + 8 + j] = static_cast<uint8_t>(val >> (8 * j));
  }
  return d;
}

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr uint8_t kSignature[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
constexpr size_t kSuperblock = 48;
constexpr int kAttrString = 256;

enum Msg : uint8_t {
  kNil = 0x00,
  kDataspace = 0x01,
  kLinkInfo = 0x02,
  kDatatype = 0x03,
  kFillValue = 0x05,
  kLink = 0x06,
  kLayout = 0x08,
  kGroupInfo = 0x0A,
  kAttribute = 0x0C,
};

struct Out {
  std::vector<uint8_t> b;
  void u8(unsigned v) { b.push_back(static_cast<uint8_t>(v)); }
  void u16(unsigned v)
  {
    u8(v & 0xff);
    u8((v >> 8) & 0xff);
  }
  void u32(uint32_t v)
  {
    for (int i = 0; i < 4; ++i) u8((v >> (8 * i)) & 0xff);
  }
  void u64(uint64_t v)
  {
    for (int i = 0; i < 8; ++i) u8(static_cast<unsigned>((v >> (8 * i)) & 0xff));
  }
  void raw(const void* p, size_t n)
  {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    b.insert(b.end(), c, c + n);
  }
};

// Datatype message bodies.
void dt_fixed(Out& o, int size, bool is_signed)
{
  o.u8(0x10);                    // version 1, class 0 (fixed-point)
  o.u8(is_signed ? 0x08 : 0x00);  // little-endian, zero padding, signedness
  o.u8(0);
  o.u8(0);
  o.u32(static_cast<uint32_t>(size));
  o.u16(0);                      // bit offset
  o.u16(static_cast<unsigned>(8 * size));  // bit precision
}

void dt_double(Out& o)
{
  o.u8(0x11);  // version 1, class 1 (floating-point)
  o.u8(0x20);  // little-endian, zero padding, mantissa normalisation: implied MSB
  o.u8(63);    // sign bit location
  o.u8(0);
  o.u32(8);
  o.u16(0);     // bit offset
  o.u16(64);    // bit precision
  o.u8(52);     // exponent location
  o.u8(11);     // exponent size
  o.u8(0);      // mantissa location
  o.u8(52);     // mantissa size
  o.u32(1023);  // exponent bias
}

void dt_string(Out& o, int size)
{
  o.u8(0x13);  // version 1, class 3 (string)
  o.u8(0x00);  // null-terminated, ASCII
  o.u8(0);
  o.u8(0);
  o.u32(static_cast<uint32_t>(size));
}

// Compound {Key: int32 at 0, Value: float64 at 8}, 16 bytes, version 1 members.
void dt_key_value(Out& o)
{
  o.u8(0x16);  // version 1, class 6 (compound)
  o.u16(2);    // members
  o.u8(0);
  o.u32(16);
  auto member = [&](const char* name, uint32_t offset, const std::function<void(Out&)>& type) {
    const size_t n = std::strlen(name) + 1;
    o.raw(name, n);
    for (size_t i = n; i % 8 != 0; ++i) o.u8(0);  // name padded to a multiple of 8
    o.u32(offset);
    o.u8(0);  // dimensionality
    o.u8(0);
    o.u8(0);
    o.u8(0);
    o.u32(0);  // dimension permutation
    o.u32(0);
    for (int i = 0; i < 4; ++i) o.u32(0);  // dimension sizes
    type(o);
  };
  member("Key", 0, [](Out& t) { dt_fixed(t, 4, true); });
  member("Value", 8, [](Out& t) { dt_double(t); });
}

void datatype(Out& o, Type t)
{
  switch (t) {
    case Type::u8: dt_fixed(o, 1, false); break;
    case Type::i8: dt_fixed(o, 1, true); break;
    case Type::i32: dt_fixed(o, 4, true); break;
    case Type::u64: dt_fixed(o, 8, false); break;
    case Type::f64: dt_double(o); break;
    case Type::key_value: dt_key_value(o); break;
  }
}

size_t elem_size(Type t)
{
  switch (t) {
    case Type::u8:
    case Type::i8: return 1;
    case Type::i32: return 4;
    case Type::u64:
    case Type::f64: return 8;
    case Type::key_value: return 16;
  }
  return 1;
}

void dataspace_simple(Out& o, uint64_t n)
{
  o.u8(2);  // version
  o.u8(1);  // rank
  o.u8(0);  // no maximum dimensions
  o.u8(1);  // simple
  o.u64(n);
}

void dataspace_scalar(Out& o)
{
  o.u8(2);
  o.u8(0);
  o.u8(0);
  o.u8(0);  // scalar
}

void message(Out& o, uint8_t type, const Out& body, uint8_t flags = 0)
{
  o.u8(type);
  o.u16(static_cast<unsigned>(body.b.size()));
  o.u8(flags);
  o.raw(body.b.data(), body.b.size());
}

// Version-2 object header around the serialised messages.
std::vector<uint8_t> object_header(const Out& msgs)
{
  Out o;
  o.raw("OHDR", 4);
  o.u8(2);     // version
  o.u8(0x02);  // chunk #0 size in 4 bytes; no times, no attribute phase values
  o.u32(static_cast<uint32_t>(msgs.b.size()));
  o.raw(msgs.b.data(), msgs.b.size());
  o.u32(lookup3(o.b.data(), o.b.size()));
  return o.b;
}

struct Node {
  const Group* g = nullptr;
  const Dataset* d = nullptr;
  uint64_t addr = 0, data_addr = 0, header_size = 0;
  std::vector<std::pair<std::string, Node*>> children;
};

Out dataset_messages(const Dataset& d, uint64_t data_addr)
{
  Out msgs, body;
  dataspace_simple(body, d.count);
  message(msgs, kDataspace, body);
  body.b.clear();
  datatype(body, d.type);
  message(msgs, kDatatype, body, 0x01);  // constant
  body.b.clear();
  body.u8(3);     // version
  body.u8(0x0A);  // allocation time late, fill value written if set, none defined
  message(msgs, kFillValue, body, 0x01);
  body.b.clear();
  body.u8(3);  // version
  body.u8(1);  // contiguous
  body.u64(d.bytes.empty() ? kUndef : data_addr);
  body.u64(d.bytes.size());
  message(msgs, kLayout, body);
  for (const auto& [name, text] : d.string_attrs) {
    Out dt, ds, a;
    dt_string(dt, kAttrString);
    dataspace_scalar(ds);
    a.u8(3);  // version
    a.u8(0);
    a.u16(static_cast<unsigned>(name.size() + 1));
    a.u16(static_cast<unsigned>(dt.b.size()));
    a.u16(static_cast<unsigned>(ds.b.size()));
    a.u8(0);  // ASCII name
    a.raw(name.c_str(), name.size() + 1);
    a.raw(dt.b.data(), dt.b.size());
    a.raw(ds.b.data(), ds.b.size());
    std::string value = text.substr(0, kAttrString - 1);
    value.resize(kAttrString, '\0');
    a.raw(value.data(), value.size());
    message(msgs, kAttribute, a);
  }
  return msgs;
}

Out group_messages(const Node& n)
{
  Out msgs, body;
  body.u8(0);  // Link Info version
  body.u8(0);  // no creation order
  body.u64(kUndef);  // fractal heap (compact storage)
  body.u64(kUndef);  // name index
  message(msgs, kLinkInfo, body);
  body.b.clear();
  body.u8(0);  // Group Info version
  body.u8(0);
  message(msgs, kGroupInfo, body);
  for (const auto& [name, child] : n.children) {
    body.b.clear();
    body.u8(1);  // Link version
    if (name.size() < 256) {
      body.u8(0x00);  // 1-byte name length, hard link
      body.u8(static_cast<unsigned>(name.size()));
    } else {
      body.u8(0x01);  // 2-byte name length
      body.u16(static_cast<unsigned>(name.size()));
    }
    body.raw(name.data(), name.size());
    body.u64(child->addr);
    message(msgs, kLink, body);
  }
  return msgs;
}

}  // namespace

std::string write_file(const std::string& path, const Group& root)
{
  std::vector<std::unique_ptr<Node>> nodes;
  std::function<Node*(const Group*, const Dataset*)> build = [&](const Group* g, const Dataset* d) {
    nodes.push_back(std::make_unique<Node>());
    Node* n = nodes.back().get();
    n->g = g;
    n->d = d;
    if (g != nullptr) {
      for (const auto& [name, child] : g->groups) n->children.emplace_back(name, build(child.get(), nullptr));
      for (const auto& [name, ds] : g->datasets) n->children.emplace_back(name, build(nullptr, &ds));
    }
    return n;
  };
  Node* top = build(&root, nullptr);
  // header sizes do not depend on addresses: size with placeholder addresses
  for (auto& n : nodes) {
    const Out m = n->g ? group_messages(*n) : dataset_messages(*n->d, 0);
    n->header_size = object_header(m).size();
  }
  // addresses in creation (pre-)order: header, then a dataset's raw data
  uint64_t addr = kSuperblock;
  for (auto& n : nodes) {
    n->addr = addr;
    addr += n->header_size;
    if (n->d != nullptr) {
      addr = (addr + 7) & ~7ull;
      n->data_addr = addr;
      addr += n->d->bytes.size();
      addr = (addr + 7) & ~7ull;
    }
  }
  const uint64_t eof = addr;
  std::vector<uint8_t> file(eof, 0);
  Out sb;
  sb.raw(kSignature, 8);
  sb.u8(2);  // superblock version
  sb.u8(8);  // size of offsets
  sb.u8(8);  // size of lengths
  sb.u8(0);  // consistency flags
  sb.u64(0);       // base address
  sb.u64(kUndef);  // superblock extension
  sb.u64(eof);
  sb.u64(top->addr);
  sb.u32(lookup3(sb.b.data(), sb.b.size()));
  std::memcpy(file.data(), sb.b.data(), sb.b.size());
  for (auto& n : nodes) {
    const Out m = n->g ? group_messages(*n) : dataset_messages(*n->d, n->data_addr);
    const std::vector<uint8_t> h = object_header(m);
    if (h.size() != n->header_size) return "internal: header size changed";
    std::memcpy(file.data() + n->addr, h.data(), h.size());
    if (n->d != nullptr && !n->d->bytes.empty())
      std::memcpy(file.data() + n->data_addr, n->d->bytes.data(), n->d->bytes.size());
  }
  const std::string tmp = path + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (f == nullptr) return "cannot create " + tmp;
  const bool ok = std::fwrite(file.data(), 1, file.size(), f) == file.size();
  if (std::fclose(f) != 0 || !ok) return "cannot write " + tmp;
  if (std::rename(tmp.c_str(), path.c_str()) != 0) return "cannot rename " + tmp;
  return "";
}

namespace {

struct In {
  const std::vector<uint8_t>& b;
  uint64_t pos;
  bool ok = true;
  bool need(uint64_t n)
  {
    if (n > b.size() || pos > b.size() - n) ok = false;  // no wrap-around for offsets read from the file
    return ok;
  }
  // Little-endian field of n <= 8 bytes (field sizes can come from the file).
  uint64_t le(int n)
  {
    if (n < 0 || n > 8) ok = false;
    if (!ok || !need(static_cast<uint64_t>(n))) return 0;
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v |= static_cast<uint64_t>(b[pos + i]) << (8 * i);
    pos += static_cast<uint64_t>(n);
    return v;
  }
  void skip(uint64_t n)
  {
    if (need(n)) pos += n;
  }
};

// [at, at + n) lies inside the file (no wrap-around for file offsets).
bool fits(const std::vector<uint8_t>& file, uint64_t at, uint64_t n)
{
  return n <= file.size() && at <= file.size() - n;
}

// Datatype at in.pos -> Type; false if not one this module writes.
bool parse_type(In& in, Type& t, bool member = false)
{
  const uint64_t start = in.pos;
  const unsigned cv = static_cast<unsigned>(in.le(1));
  const unsigned f0 = static_cast<unsigned>(in.le(1));
  in.le(2);
  const uint64_t size = in.le(4);
  if (!in.ok) return false;
  const unsigned cls = cv & 0x0f;
  if (cls == 0) {
    in.le(4);
    const bool sgn = (f0 & 0x08) != 0;
    if (size == 1) t = sgn ? Type::i8 : Type::u8;
    else if (size == 4 && sgn) t = Type::i32;
    else if (size == 8 && !sgn) t = Type::u64;
    else return false;
    return in.ok;
  }
  if (cls == 1) {
    in.skip(12);
    if (size != 8) return false;
    t = Type::f64;
    return in.ok;
  }
  if (cls == 6 && (cv >> 4) == 1 && size == 16 && !member) {
    // version-1 compound: two members Key (int32 at 0), Value (float64 at 8)
    const unsigned members = f0 | (static_cast<unsigned>(in.b[start + 2]) << 8);
    if (members != 2) return false;
    for (unsigned m = 0; m < 2; ++m) {
      std::string name;
      while (in.need(1) && in.b[in.pos] != 0) name.push_back(static_cast<char>(in.b[in.pos++]));
      const size_t padded = (name.size() + 1 + 7) / 8 * 8;
      in.pos += padded - name.size();
      const uint64_t off = in.le(4);
      in.skip(28);
      Type mt;
      if (!parse_type(in, mt, true)) return false;
      if (m == 0 && (name != "Key" || off != 0 || mt != Type::i32)) return false;
      if (m == 1 && (name != "Value" || off != 8 || mt != Type::f64)) return false;
    }
    t = Type::key_value;
    return in.ok;
  }
  return false;
}

// A header message: type and the byte range of its body.
struct HMsg {
  unsigned type;
  uint64_t body, size;
};

constexpr unsigned kContinuation = 0x10;
constexpr unsigned kSymbolTable = 0x11;

uint32_t le32_at(const std::vector<uint8_t>& f, uint64_t a)
{
  return static_cast<uint32_t>(f[a]) | static_cast<uint32_t>(f[a + 1]) << 8 | static_cast<uint32_t>(f[a + 2]) << 16 |
         static_cast<uint32_t>(f[a + 3]) << 24;
}

// The messages of the object header at addr, version 2 ("OHDR", IV.A.1.b,
// continuation blocks "OCHK") or version 1 (IV.A.1.a: no signature, 8-byte
// aligned messages, continuation blocks of bare messages), in order.
std::string header_messages(const std::vector<uint8_t>& file, uint64_t addr, std::vector<HMsg>& out)
{
  out.clear();
  if (!fits(file, addr, 16)) return "object header address";
  std::vector<std::pair<uint64_t, uint64_t>> blocks;  // message ranges still to read
  const bool v2 = std::memcmp(file.data() + addr, "OHDR", 4) == 0;
  unsigned crt = 0;
  if (v2) {
    In in{file, addr + 4};
    const unsigned version = static_cast<unsigned>(in.le(1));
    const unsigned flags = static_cast<unsigned>(in.le(1));
    if (version != 2) return "object header version";
    if (flags & 0x20) in.skip(16);
    if (flags & 0x10) in.le(4);
    const uint64_t chunk = in.le(1 << (flags & 3));
    crt = (flags & 0x04) ? 2 : 0;
    if (!in.ok || !fits(file, in.pos, chunk) || !fits(file, in.pos + chunk, 4)) return "object header size";
    const uint64_t msg_start = in.pos, msg_end = in.pos + chunk;
    if (lookup3(file.data() + addr, msg_end - addr) != le32_at(file, msg_end)) return "object header checksum";
    blocks.emplace_back(msg_start, msg_end);
  } else {
    In in{file, addr};
    if (in.le(1) != 1) return "object header version";
    in.le(1);
    in.le(2);  // message count (the blocks' sizes bound the reading)
    in.le(4);  // reference count
    const uint64_t size = in.le(4);
    if (!in.ok || !fits(file, addr + 16, size)) return "object header size";
    blocks.emplace_back(addr + 16, addr + 16 + size);
  }
  for (size_t bi = 0; bi < blocks.size(); ++bi) {
    if (bi > 64) return "too many continuation blocks";
    auto [pos, end] = blocks[bi];
    if (v2 && bi > 0) {  // "OCHK", messages, checksum
      if (end < pos + 8 || std::memcmp(file.data() + pos, "OCHK", 4) != 0) return "continuation block";
      if (lookup3(file.data() + pos, end - 4 - pos) != le32_at(file, end - 4)) return "continuation checksum";
      pos += 4;
      end -= 4;
    }
    In in{file, pos};
    const uint64_t head = v2 ? 4 + crt : 8;
    while (in.pos + head <= end) {
      unsigned type;
      uint64_t size;
      if (v2) {
        type = static_cast<unsigned>(in.le(1));
        size = in.le(2);
        in.le(1);
        in.le(static_cast<int>(crt));
      } else {
        type = static_cast<unsigned>(in.le(2));
        size = in.le(2);
        in.le(1);
        in.le(3);
      }
      const uint64_t body = in.pos;
      if (!in.ok || body + size > end) return "message size";
      if (type == kContinuation) {
        In c{file, body};
        const uint64_t at = c.le(8), len = c.le(8);
        if (!c.ok || !fits(file, at, len)) return "continuation address";
        blocks.emplace_back(at, at + len);
      } else if (type != kNil) {
        out.push_back({type, body, size});
      }
      in.pos = body + size;
    }
  }
  return "";
}

// Links of an old-style group (III.A.1 version-1 B-tree of group nodes,
// III.B symbol table nodes, III.D local heap for the names).
// Limits that bound the work on a damaged or hostile file (nodes shared
// between parents, links back to an ancestor): far above what the programs
// write (a pre-run file of 1000 samples holds ~10^5 objects).
constexpr size_t kMaxNodes = size_t{1} << 20;
constexpr size_t kMaxLinks = size_t{1} << 22;

std::string symbol_table_links(const std::vector<uint8_t>& file, uint64_t btree, uint64_t heap,
                               std::vector<std::pair<std::string, uint64_t>>& links, int depth, int expect_level,
                               size_t& nodes)
{
  if (depth > 32) return "B-tree too deep";
  if (++nodes > kMaxNodes) return "too many B-tree nodes";
  if (!fits(file, heap, 32) || std::memcmp(file.data() + heap, "HEAP", 4) != 0) return "local heap";
  In h{file, heap + 8};
  const uint64_t seg_size = h.le(8);
  h.le(8);
  const uint64_t seg = h.le(8);
  if (!h.ok || !fits(file, seg, seg_size)) return "local heap segment";
  if (!fits(file, btree, 24) || std::memcmp(file.data() + btree, "TREE", 4) != 0) return "group B-tree";
  In t{file, btree + 4};
  const unsigned type = static_cast<unsigned>(t.le(1));
  const unsigned level = static_cast<unsigned>(t.le(1));
  const uint64_t used = t.le(2);
  t.le(8);
  t.le(8);
  if (type != 0) return "B-tree node type";
  if (expect_level >= 0 && static_cast<int>(level) != expect_level) return "B-tree level";
  for (uint64_t k = 0; k < used; ++k) {
    t.le(8);  // key: heap offset of the largest name in the child
    const uint64_t child = t.le(8);
    if (!t.ok) return "B-tree node";
    if (level > 0) {
      const std::string err = symbol_table_links(file, child, heap, links, depth + 1, static_cast<int>(level) - 1, nodes);
      if (!err.empty()) return err;
      continue;
    }
    if (!fits(file, child, 8) || std::memcmp(file.data() + child, "SNOD", 4) != 0) return "symbol table node";
    In sn{file, child + 4};
    if (sn.le(1) != 1) return "symbol table node version";
    sn.le(1);
    const uint64_t nsym = sn.le(2);
    for (uint64_t e = 0; e < nsym; ++e) {
      const uint64_t name_off = sn.le(8);
      const uint64_t obj = sn.le(8);
      sn.le(4);
      sn.le(4);
      sn.skip(16);
      if (!sn.ok || name_off >= seg_size) return "symbol table entry";
      if (links.size() >= kMaxLinks) return "too many links";
      const char* nm = reinterpret_cast<const char*>(file.data() + seg + name_off);
      links.emplace_back(std::string(nm, strnlen(nm, seg_size - name_off)), obj);
    }
  }
  return "";
}

// Work bounds of one parse: every object header takes at least 16 bytes of
// the file and every dataset's bytes are stored once, so a file whose links
// reach more objects or more data than that shares objects between parents
// (or links back to an ancestor) and is refused.
struct Budget {
  uint64_t objects, bytes;
  std::vector<uint64_t> ancestors;
};

std::string parse_object(const std::vector<uint8_t>& file, uint64_t addr, Group* g, Dataset* d, int depth,
                         bool* is_group, Budget& budget)
{
  if (depth > 64) return "nesting too deep";
  if (budget.objects == 0) return "objects shared between groups";
  --budget.objects;
  std::vector<HMsg> msgs;
  std::string herr = header_messages(file, addr, msgs);
  if (!herr.empty()) return herr;
  std::vector<std::pair<std::string, uint64_t>> links;
  bool has_layout = false;
  Type type = Type::u8;
  uint64_t count = 0, data_addr = kUndef, data_size = 0;
  std::vector<uint8_t> compact;
  bool is_compact = false;
  std::map<std::string, std::string> attrs;
  for (const HMsg& msg : msgs) {
    In m{file, msg.body};
    switch (msg.type) {
      case kLink: {
        const unsigned lv = static_cast<unsigned>(m.le(1));
        const unsigned lf = static_cast<unsigned>(m.le(1));
        if (lv != 1) return "link version";
        unsigned ltype = 0;
        if (lf & 0x08) ltype = static_cast<unsigned>(m.le(1));
        if (lf & 0x04) m.le(8);
        if (lf & 0x10) m.le(1);
        const uint64_t nlen = m.le(1 << (lf & 3));
        if (!m.need(nlen)) return "link name";
        std::string name(reinterpret_cast<const char*>(file.data() + m.pos), nlen);
        m.pos += nlen;
        if (ltype != 0) return "soft or external link";
        links.emplace_back(name, m.le(8));
        break;
      }
      case kSymbolTable: {
        const uint64_t bt = m.le(8), hp = m.le(8);
        if (!m.ok) break;
        size_t nodes = 0;
        const std::string err = symbol_table_links(file, bt, hp, links, 0, -1, nodes);
        if (!err.empty()) return err;
        break;
      }
      case kDataspace: {
        const unsigned sv = static_cast<unsigned>(m.le(1));
        const unsigned rank = static_cast<unsigned>(m.le(1));
        m.le(1);  // flags
        if (sv == 1) {
          m.le(5);  // reserved
        } else if (sv == 2) {
          m.le(1);  // type
        } else {
          return "dataspace version";
        }
        count = 1;
        for (unsigned r = 0; r < rank; ++r) {
          const uint64_t dim = m.le(8);
          if (dim != 0 && count > ~uint64_t{0} / dim) return "dataspace size";
          count *= dim;
        }
        break;
      }
      case kDatatype:
        if (!parse_type(m, type)) return "unsupported datatype";
        break;
      case kLayout: {
        const unsigned lv = static_cast<unsigned>(m.le(1));
        const unsigned cls = static_cast<unsigned>(m.le(1));
        if (lv != 3 || cls > 1) return "unsupported layout";
        if (cls == 1) {
          data_addr = m.le(8);
          data_size = m.le(8);
        } else {  // compact: the data is in the message
          data_size = m.le(2);
          if (!m.need(data_size)) return "compact data";
          compact.assign(file.begin() + static_cast<long>(m.pos), file.begin() + static_cast<long>(m.pos + data_size));
          is_compact = true;
        }
        has_layout = true;
        break;
      }
      case kAttribute: {
        const unsigned av = static_cast<unsigned>(m.le(1));
        m.le(1);
        const uint64_t nsz = m.le(2), tsz = m.le(2), ssz = m.le(2);
        if (av < 1 || av > 3) return "attribute version";
        if (av == 3) m.le(1);
        auto pad = [av](uint64_t n) { return av == 1 ? (n + 7) / 8 * 8 : n; };
        if (!m.need(pad(nsz) + pad(tsz) + pad(ssz))) return "attribute";
        std::string name(reinterpret_cast<const char*>(file.data() + m.pos), strnlen(reinterpret_cast<const char*>(
                                                                                   file.data() + m.pos), nsz));
        m.pos += pad(nsz);
        const uint64_t dt = m.pos;
        m.pos += pad(tsz) + pad(ssz);
        if (tsz >= 8 && (file[dt] & 0x0f) == 3) {
          const uint64_t len = static_cast<uint64_t>(file[dt + 4]) | static_cast<uint64_t>(file[dt + 5]) << 8;
          if (m.need(len)) {
            std::string v(reinterpret_cast<const char*>(file.data() + m.pos), len);
            v.resize(std::strlen(v.c_str()));
            attrs[name] = v;
          }
        }
        break;
      }
      default:
        break;
    }
    if (!m.ok) return "truncated message";
  }
  *is_group = !has_layout;
  if (has_layout) {
    if (d == nullptr) return "dataset where a group was expected";
    d->type = type;
    d->count = count;
    d->string_attrs = attrs;
    const uint64_t esize = elem_size(type);
    if (data_size % esize != 0 || count != data_size / esize) return "dataset size";
    if (data_size > budget.bytes) return "data shared between datasets";
    budget.bytes -= data_size;
    if (is_compact) {
      d->bytes = compact;
    } else if (data_size > 0) {
      if (data_addr == kUndef || data_addr + data_size > file.size()) return "dataset address";
      d->bytes.assign(file.begin() + static_cast<long>(data_addr), file.begin() + static_cast<long>(data_addr + data_size));
    }
    return "";
  }
  if (g == nullptr) return "group where a dataset was expected";
  for (const auto& [name, child] : links) {
    Group sub;
    Dataset ds;
    bool child_group = false;
    // a child is a dataset exactly when its header has a layout message
    if (std::find(budget.ancestors.begin(), budget.ancestors.end(), child) != budget.ancestors.end())
      return name + ": link to an enclosing group";
    budget.ancestors.push_back(addr);
    std::string err = parse_object(file, child, &sub, &ds, depth + 1, &child_group, budget);
    budget.ancestors.pop_back();
    if (!err.empty()) return name + ": " + err;
    if (child_group) g->groups[name] = std::make_unique<Group>(std::move(sub));
    else g->datasets[name] = std::move(ds);
  }
  return "";
}

}  // namespace

std::string read_file(const std::string& path, Group& root)
{
  FILE* f = std::fopen(path.c_str(), "rb");
  if (f == nullptr) return "cannot open " + path;
  std::vector<uint8_t> file;
  uint8_t buf[65536];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) file.insert(file.end(), buf, buf + n);
  std::fclose(f);
  if (file.size() < kSuperblock || std::memcmp(file.data(), kSignature, 8) != 0) return "not an HDF5 file";
  uint64_t root_addr = 0;
  if (file[8] == 0 || file[8] == 1) {
    // II.A.1 superblock version 0/1 (libhdf5's default): sizes at 13-14,
    // base address at 24 (28 for version 1), then free space, end of file and
    // driver addresses, then the root group's symbol table entry
    if (file[13] != 8 || file[14] != 8) return "offset/length sizes";
    const uint64_t base_at = file[8] == 0 ? 24 : 28;
    if (file.size() < base_at + 32 + 40) return "superblock size";
    In in{file, base_at};
    if (in.le(8) != 0) return "base address";
    in.le(8);
    in.le(8);
    in.le(8);
    in.le(8);  // root entry: link name offset
    root_addr = in.le(8);
  } else if (file[8] == 2 || file[8] == 3) {
    if (file[9] != 8 || file[10] != 8) return "offset/length sizes";
    In in{file, 12};
    in.le(8);
    in.le(8);
    in.le(8);
    root_addr = in.le(8);
    const uint32_t sum = static_cast<uint32_t>(in.le(4));
    if (lookup3(file.data(), 44) != sum) return "superblock checksum";
  } else {
    return "superblock version " + std::to_string(file[8]);
  }
  root.groups.clear();
  root.datasets.clear();
  bool is_group = false;
  Dataset unused;
  Budget budget{file.size() / 16 + 1, file.size(), {}};
  std::string err = parse_object(file, root_addr, &root, &unused, 0, &is_group, budget);
  if (err.empty() && !is_group) err = "root is not a group";
  return err;
}

}  // namespace wlg::h5

// ------------------------------------------------------------------ C ABI --

#include "../../include/wlg.h"
#include "wlg_internal.h"

namespace {

// Object at a '/'-separated path below the root: a group or a dataset.
std::string find(const wlg::h5::Group& root, const char* path, const wlg::h5::Group** g, const wlg::h5::Dataset** d)
{
  *g = &root;
  *d = nullptr;
  std::string p = path == nullptr ? "" : path;
  size_t i = 0;
  while (i < p.size()) {
    size_t j = p.find('/', i);
    if (j == std::string::npos) j = p.size();
    const std::string part = p.substr(i, j - i);
    i = j + 1;
    if (part.empty()) continue;
    if (*d != nullptr || *g == nullptr) return "not found";
    auto gi = (*g)->groups.find(part);
    if (gi != (*g)->groups.end()) {
      *g = gi->second.get();
      continue;
    }
    auto di = (*g)->datasets.find(part);
    if (di == (*g)->datasets.end()) return "not found";
    *d = &di->second;
    *g = nullptr;
  }
  return "";
}

}  // namespace

extern "C" {

unsigned int wlg_h5_lookup3(const void* data, size_t n, unsigned int init)
{
  return wlg::h5::lookup3(static_cast<const uint8_t*>(data), n, init);
}

wlg_status wlg_h5_list(const char* file, const char* group, char* names, size_t cap)
{
  return wlg::guarded([&]() -> wlg_status {
    if (file == nullptr || names == nullptr || cap == 0) return WLG_ERR_INVALID;
    wlg::h5::Group root;
    if (!wlg::h5::read_file(file, root).empty()) return WLG_ERR_INVALID;
    const wlg::h5::Group* g;
    const wlg::h5::Dataset* d;
    if (!find(root, group, &g, &d).empty() || g == nullptr) return WLG_ERR_INVALID;
    std::string out;
    for (const auto& [k, v] : g->groups) out += k + "/\n";
    for (const auto& [k, v] : g->datasets) out += k + "\n";
    if (out.size() + 1 > cap) return WLG_ERR_CAPACITY;
    std::memcpy(names, out.c_str(), out.size() + 1);
    return WLG_OK;
  });
}

wlg_status wlg_h5_read(const char* file, const char* dataset, int* type, unsigned long long* count, void* buf,
                       unsigned long long cap_bytes)
{
  return wlg::guarded([&]() -> wlg_status {
    if (file == nullptr || dataset == nullptr || type == nullptr || count == nullptr) return WLG_ERR_INVALID;
    wlg::h5::Group root;
    if (!wlg::h5::read_file(file, root).empty()) return WLG_ERR_INVALID;
    const wlg::h5::Group* g;
    const wlg::h5::Dataset* d;
    if (!find(root, dataset, &g, &d).empty() || d == nullptr) return WLG_ERR_INVALID;
    *type = static_cast<int>(d->type);
    *count = d->count;
    if (buf != nullptr) {
      if (d->bytes.size() > cap_bytes) return WLG_ERR_CAPACITY;
      std::memcpy(buf, d->bytes.data(), d->bytes.size());
    }
    return WLG_OK;
  });
}

wlg_status wlg_h5_attribute(const char* file, const char* dataset, const char* name, char* out, size_t cap)
{
  return wlg::guarded([&]() -> wlg_status {
    if (file == nullptr || dataset == nullptr || name == nullptr || out == nullptr || cap == 0) return WLG_ERR_INVALID;
    wlg::h5::Group root;
    if (!wlg::h5::read_file(file, root).empty()) return WLG_ERR_INVALID;
    const wlg::h5::Group* g;
    const wlg::h5::Dataset* d;
    if (!find(root, dataset, &g, &d).empty() || d == nullptr) return WLG_ERR_INVALID;
    auto it = d->string_attrs.find(name);
    if (it == d->string_attrs.end()) return WLG_ERR_INVALID;
    if (it->second.size() + 1 > cap) return WLG_ERR_CAPACITY;
    std::memcpy(out, it->second.c_str(), it->second.size() + 1);
    return WLG_OK;
  });
}

}  // extern "C"
