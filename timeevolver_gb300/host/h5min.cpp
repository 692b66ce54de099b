// h5min.cpp -- HDF5 writer for result files (see h5min.h).  Field layouts
// follow the HDF5 file format specification: superblock version 0, B-tree
// version 1 (group nodes), symbol-table node version 1, local heap version 0,
// object header version 1 with messages 0x0001 dataspace (v1), 0x0003
// datatype (v1), 0x0005 fill value (v2), 0x0008 layout (v3, contiguous),
// 0x0012 modification time (v1), 0x000C attribute (v1), 0x0011 symbol table.
#include "h5min.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>

namespace h5min {
namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kLeafK = 4;       // default group leaf node K (raised for many datasets)
constexpr int kInternalK = 16;  // default group internal node K

class Buf {
 public:
  std::vector<uint8_t> b;
  void u8(uint64_t v) { b.push_back((uint8_t)v); }
  void le(uint64_t v, int n) {
    for (int i = 0; i < n; ++i) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void bytes(const void* p, size_t n) {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    b.insert(b.end(), c, c + n);
  }
  void pad8() {
    while (b.size() % 8) b.push_back(0);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  size_t size() const { return b.size(); }
  void put(size_t at, uint64_t v, int n) {
    for (int i = 0; i < n; ++i) b[at + i] = (uint8_t)(v >> (8 * i));
  }
};

uint64_t align8(uint64_t v) { return (v + 7) & ~7ull; }

// Datatype message bodies (unpadded sizes 20, 12).
void dt_double(Buf& o) {
  o.u8(0x11);  // class 1 (floating point), version 1
  o.u8(0x20);  // little endian, no padding bits, mantissa normalisation: implied msb
  o.u8(63);    // sign bit location
  o.u8(0);
  o.le(8, 4);   // size
  o.le(0, 2);   // bit offset
  o.le(64, 2);  // precision
  o.u8(52);     // exponent location
  o.u8(11);     // exponent size
  o.u8(0);      // mantissa location
  o.u8(52);     // mantissa size
  o.le(1023, 4);  // exponent bias
}
void dt_int(Buf& o, int size, bool is_signed) {
  o.u8(0x10);  // class 0 (fixed point), version 1
  o.u8(is_signed ? 0x08 : 0x00);  // little endian, two's complement when signed
  o.u8(0);
  o.u8(0);
  o.le((uint64_t)size, 4);
  o.le(0, 2);             // bit offset
  o.le(8 * size, 2);      // precision
}

// Dataspace message body: version 1, rank 1, maximum dimension present.
void dataspace1(Buf& o, uint64_t n) {
  o.u8(1);
  o.u8(1);
  o.u8(1);
  o.zeros(5);
  o.le(n, 8);
  o.le(n, 8);
}

void message(Buf& o, int type, int flags, const Buf& body) {
  o.le((uint64_t)type, 2);
  o.le(align8(body.size()), 2);
  o.u8((uint64_t)flags);
  o.zeros(3);
  o.bytes(body.b.data(), body.size());
  o.pad8();
}

Buf attribute_body(const Attribute& a) {
  Buf dt, ds, o;
  if (a.is_double)
    dt_double(dt);
  else
    dt_int(dt, 4, true);
  dataspace1(ds, 1);
  o.u8(1);  // version
  o.u8(0);
  o.le(a.name.size() + 1, 2);
  o.le(dt.size(), 2);
  o.le(ds.size(), 2);
  o.bytes(a.name.c_str(), a.name.size() + 1);
  o.pad8();
  o.bytes(dt.b.data(), dt.size());
  o.pad8();
  o.bytes(ds.b.data(), ds.size());
  o.pad8();
  if (a.is_double) {
    uint64_t bits;
    std::memcpy(&bits, &a.d, 8);
    o.le(bits, 8);
  } else {
    o.le((uint32_t)a.i, 4);
  }
  return o;
}

// The object header of a dataset whose values start at data_addr.
Buf dataset_header(const Dataset& d, uint64_t data_addr, uint32_t mtime) {
  Buf msgs;
  int count = 0;
  {
    Buf b;
    dataspace1(b, d.count);
    message(msgs, 0x0001, 0, b);
    ++count;
  }
  {
    Buf b;
    if (d.type == Type::F64)
      dt_double(b);
    else
      dt_int(b, 8, false);
    message(msgs, 0x0003, 1, b);  // constant
    ++count;
  }
  {
    Buf b;  // version 2; allocation late, fill written if set, fill value defined (default)
    b.u8(2);
    b.u8(2);
    b.u8(2);
    b.u8(1);
    b.le(0, 4);
    message(msgs, 0x0005, 1, b);
    ++count;
  }
  {
    Buf b;
    b.u8(3);  // version 3
    b.u8(1);  // contiguous
    b.le(data_addr, 8);
    b.le(d.bytes.size(), 8);
    message(msgs, 0x0008, 0, b);
    ++count;
  }
  {
    Buf b;
    b.u8(1);
    b.zeros(3);
    b.le(mtime, 4);
    message(msgs, 0x0012, 0, b);
    ++count;
  }
  for (const Attribute& a : d.attributes) {
    message(msgs, 0x000C, 0, attribute_body(a));
    ++count;
  }
  Buf h;
  h.u8(1);  // version 1
  h.u8(0);
  h.le((uint64_t)count, 2);
  h.le(1, 4);             // reference count
  h.le(msgs.size(), 4);   // header data size
  h.zeros(4);             // alignment of the messages
  h.bytes(msgs.b.data(), msgs.size());
  return h;
}

}  // namespace

void File::add(const std::string& name, const double* values, uint64_t count, std::vector<Attribute> attrs) {
  Dataset d;
  d.name = name;
  d.type = Type::F64;
  d.count = count;
  d.bytes.resize(8 * count);
  for (uint64_t i = 0; i < count; ++i) {
    uint64_t bits;
    std::memcpy(&bits, values + i, 8);
    for (int k = 0; k < 8; ++k) d.bytes[8 * i + k] = (uint8_t)(bits >> (8 * k));
  }
  d.attributes = std::move(attrs);
  sets_.push_back(std::move(d));
}

void File::add(const std::string& name, const uint64_t* values, uint64_t count, std::vector<Attribute> attrs) {
  Dataset d;
  d.name = name;
  d.type = Type::U64;
  d.count = count;
  d.bytes.resize(8 * count);
  for (uint64_t i = 0; i < count; ++i)
    for (int k = 0; k < 8; ++k) d.bytes[8 * i + k] = (uint8_t)(values[i] >> (8 * k));
  d.attributes = std::move(attrs);
  sets_.push_back(std::move(d));
}

void File::write(const std::string& path, uint32_t mtime) const {
  // links in name order (byte-wise, as the B-tree's keys compare)
  std::vector<size_t> order(sets_.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return sets_[a].name < sets_[b].name; });
  for (size_t i = 1; i < order.size(); ++i)
    if (sets_[order[i]].name == sets_[order[i - 1]].name)
      throw std::runtime_error("h5min: duplicate dataset name " + sets_[order[i]].name);
  for (const Dataset& d : sets_)
    if (d.name.empty() || d.name.find('/') != std::string::npos)
      throw std::runtime_error("h5min: invalid dataset name '" + d.name + "'");
  // one symbol-table node holds every link: leaf K >= ceil(links / 2)
  const int leaf_k = std::max<int>(kLeafK, (int)((sets_.size() + 1) / 2));

  // local heap data: offset 0 is the empty name, then the link names
  Buf heap;
  heap.zeros(8);
  std::vector<uint64_t> name_off(sets_.size());
  for (size_t i : order) {
    name_off[i] = heap.size();
    heap.bytes(sets_[i].name.c_str(), sets_[i].name.size() + 1);
    heap.pad8();
  }

  const uint64_t a_root = 96, root_size = 16 + 8 + 16;
  const uint64_t a_btree = a_root + root_size;
  const uint64_t btree_size = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
  const uint64_t a_heap = a_btree + btree_size, a_heap_data = a_heap + 32;
  const uint64_t a_snod = a_heap_data + heap.size();
  const uint64_t snod_size = 8 + 2 * (uint64_t)leaf_k * 40;
  uint64_t at = a_snod + snod_size;
  std::vector<uint64_t> hdr_addr(sets_.size());
  std::vector<Buf> headers(sets_.size());
  for (size_t i = 0; i < sets_.size(); ++i) {
    // the header's size does not depend on the data address
    const uint64_t hsize = dataset_header(sets_[i], 0, mtime).size();
    hdr_addr[i] = at;
    headers[i] = dataset_header(sets_[i], at + hsize, mtime);
    at = align8(at + hsize + sets_[i].bytes.size());
  }
  const uint64_t eof = at;

  Buf f;
  // superblock version 0
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  f.bytes(sig, 8);
  f.u8(0);  // superblock version
  f.u8(0);  // free-space storage version
  f.u8(0);  // root group symbol table entry version
  f.u8(0);
  f.u8(0);  // shared header message format version
  f.u8(8);  // size of offsets
  f.u8(8);  // size of lengths
  f.u8(0);
  f.le((uint64_t)leaf_k, 2);
  f.le(kInternalK, 2);
  f.le(0, 4);  // file consistency flags
  f.le(0, 8);  // base address
  f.le(kUndef, 8);  // free-space info
  f.le(eof, 8);
  f.le(kUndef, 8);  // driver information
  // root group symbol table entry: name offset, header, cache type 1 (B-tree, heap)
  f.le(0, 8);
  f.le(a_root, 8);
  f.le(1, 4);
  f.le(0, 4);
  f.le(a_btree, 8);
  f.le(a_heap, 8);
  // root object header: one symbol-table message
  f.u8(1);
  f.u8(0);
  f.le(1, 2);
  f.le(1, 4);
  f.le(24, 4);
  f.zeros(4);
  {
    Buf b;
    b.le(a_btree, 8);
    b.le(a_heap, 8);
    message(f, 0x0011, 0, b);
  }
  // B-tree node: group, leaf level, one child (the symbol-table node) keyed by
  // the empty name and the last link name
  const uint8_t tree[4] = {'T', 'R', 'E', 'E'};
  f.bytes(tree, 4);
  f.u8(0);
  f.u8(0);
  f.le(sets_.empty() ? 0 : 1, 2);
  f.le(kUndef, 8);
  f.le(kUndef, 8);
  const size_t keys_at = f.size();
  f.zeros(btree_size - 24);
  if (!sets_.empty()) {
    f.put(keys_at, 0, 8);
    f.put(keys_at + 8, a_snod, 8);
    f.put(keys_at + 16, name_off[order.back()], 8);
  }
  // local heap
  const uint8_t hp[4] = {'H', 'E', 'A', 'P'};
  f.bytes(hp, 4);
  f.u8(0);
  f.zeros(3);
  f.le(heap.size(), 8);
  f.le(kUndef, 8);  // no free block
  f.le(a_heap_data, 8);
  f.bytes(heap.b.data(), heap.size());
  // symbol-table node
  const uint8_t sn[4] = {'S', 'N', 'O', 'D'};
  f.bytes(sn, 4);
  f.u8(1);
  f.u8(0);
  f.le(sets_.size(), 2);
  for (size_t i : order) {
    f.le(name_off[i], 8);
    f.le(hdr_addr[i], 8);
    f.le(0, 4);  // no cached data
    f.le(0, 4);
    f.zeros(16);
  }
  f.zeros(40 * (2 * (uint64_t)leaf_k - sets_.size()));
  // dataset headers and values
  for (size_t i = 0; i < sets_.size(); ++i) {
    if (f.size() != hdr_addr[i]) throw std::runtime_error("h5min: layout error");
    f.bytes(headers[i].b.data(), headers[i].size());
    f.bytes(sets_[i].bytes.data(), sets_[i].bytes.size());
    f.pad8();
  }
  if (f.size() != eof) throw std::runtime_error("h5min: layout error");
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) throw std::runtime_error("h5min: cannot open " + path);
  const size_t wr = std::fwrite(f.b.data(), 1, f.size(), fp);
  const int cl = std::fclose(fp);
  if (wr != f.size() || cl != 0) throw std::runtime_error("h5min: write error on " + path);
}

}  // namespace h5min
