// fv_h5.cpp -- the reference's HDF5 snapshot file, written without an HDF5
// library (fv_h5_save).
//
// IOManager::saveSolution (IOManager.h:88-192) writes, through HighFive,
// <filename_out>.h5 holding: root attributes Ntx, Nty, Ntz, Nx, Ny, Nz, ibeg,
// iend, jbeg, jend, kbeg, kend (int) and problem (string); datasets x, y, z
// (vertex coordinates, (Nz+1)(Ny+1)(Nx+1) doubles, k/j/i order); and per save
// a group ite_<n> with datasets rho, u, v, w, prs ([Nz][Ny][Nx] doubles) and
// a time attribute (double).  The file is created at iteration 0 and opened
// read-write for each later save.
//
// This file writes that layout in the original HDF5 file format (HDF5 File
// Format Specification: superblock version 0, version-1 object headers,
// groups as symbol tables -- a version-1 B-tree of symbol-table nodes plus a
// local heap of names -- and contiguous datasets), the format libhdf5 writes
// by default, which every HDF5 reader (h5py, HighFive, ParaView, VisIt)
// opens.  Every dataset and group is written once where the file ends.  The
// root group's symbol table (name heap, nodes and B-tree), which grows by
// one entry per save, lives in a region reserved for a capacity of entries
// (twice what it holds when the region is made): a later save rewrites the
// table in that region while it fits, else reserves a region twice as large
// at the end of the file, then points the root group's symbol-table message
// and the superblock at the new table.  The capacity is read back from the
// name heap's size, whose unused tail is one free block.  Little-endian
// byte order throughout; offsets and lengths are 8 bytes.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fv3d_gb300.h"

namespace {

constexpr uint64_t kUndef = ~0ull;        // the undefined address
constexpr uint64_t kHeapFreeNull = 1;     // end of a local heap's free list
constexpr int kLeafK = 4;                 // symbol-table node: up to 2K = 8 entries
constexpr int kNodeK = 16;                // group B-tree node: up to 2K = 32 children
constexpr int kEntryBytes = 40;           // symbol-table entry with 8-byte offsets
constexpr int kSnodBytes = 8 + 2 * kLeafK * kEntryBytes;
constexpr int kTreeBytes = 24 + (2 * kNodeK + 1) * 8 + 2 * kNodeK * 8;
constexpr uint64_t kSuperblockBytes = 96;
constexpr uint64_t kRootEntryAt = 56;     // root symbol-table entry within the superblock

enum : uint16_t {
  MSG_DATASPACE = 0x1, MSG_DATATYPE = 0x3, MSG_FILL = 0x5, MSG_LAYOUT = 0x8,
  MSG_ATTRIBUTE = 0xC, MSG_SYMBOL_TABLE = 0x11
};

struct Bytes {
  std::vector<uint8_t> b;
  void u8(unsigned v) { b.push_back((uint8_t)v); }
  void u16(unsigned v) { for (int i = 0; i < 2; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
  void u32(uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
  void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
  void raw(const void* p, size_t n) { b.insert(b.end(), (const uint8_t*)p, (const uint8_t*)p + n); }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void pad8() { while (b.size() % 8) b.push_back(0); }
  size_t size() const { return b.size(); }
};

uint64_t Rd64(const uint8_t* p) {
  uint64_t v = 0;
  for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
  return v;
}
unsigned Rd16(const uint8_t* p) { return p[0] | (p[1] << 8); }

// ---- messages ---------------------------------------------------------

struct Msg {
  uint16_t type;
  uint8_t flags;
  Bytes data;  // padded to 8 bytes when the header is assembled
};

Bytes DataspaceBody(const std::vector<uint64_t>& dims) {  // version 1; rank 0 = scalar
  Bytes d;
  d.u8(1);
  d.u8((unsigned)dims.size());
  d.u8(0);  // no maximum dimensions
  d.zeros(5);
  for (uint64_t n : dims) d.u64(n);
  return d;
}

Bytes DoubleType() {  // IEEE binary64, little-endian
  Bytes d;
  d.u8(0x11);  // version 1, class 1 (floating point)
  d.u8(0x20);  // implied leading mantissa bit
  d.u8(63);    // sign bit position
  d.u8(0);
  d.u32(8);
  d.u16(0);    // bit offset
  d.u16(64);   // precision
  d.u8(52);    // exponent position
  d.u8(11);    // exponent size
  d.u8(0);     // mantissa position
  d.u8(52);    // mantissa size
  d.u32(1023); // exponent bias
  return d;
}

Bytes Int32Type() {  // signed 32-bit little-endian
  Bytes d;
  d.u8(0x10);  // version 1, class 0 (fixed point)
  d.u8(0x08);  // signed
  d.u8(0);
  d.u8(0);
  d.u32(4);
  d.u16(0);
  d.u16(32);
  return d;
}

Bytes StringType(uint32_t n) {  // fixed-length ASCII, NUL-terminated
  Bytes d;
  d.u8(0x13);  // version 1, class 3 (string)
  d.u8(0);
  d.u8(0);
  d.u8(0);
  d.u32(n);
  return d;
}

Msg Attribute(const std::string& name, const Bytes& type, const void* value, size_t nbytes) {
  Msg m{MSG_ATTRIBUTE, 0, {}};
  const Bytes space = DataspaceBody({});
  Bytes& d = m.data;
  d.u8(1);
  d.u8(0);
  d.u16((unsigned)name.size() + 1);
  d.u16((unsigned)type.size());
  d.u16((unsigned)space.size());
  d.raw(name.c_str(), name.size() + 1);
  d.pad8();
  d.raw(type.b.data(), type.size());
  d.pad8();
  d.raw(space.b.data(), space.size());
  d.pad8();
  d.raw(value, nbytes);
  return m;
}

Msg SymbolTable(uint64_t btree, uint64_t heap) {
  Msg m{MSG_SYMBOL_TABLE, 1, {}};
  m.data.u64(btree);
  m.data.u64(heap);
  return m;
}

// A version-1 object header holding `msgs`; *offsets receives each
// message's data offset within the header.
Bytes ObjectHeader(std::vector<Msg> msgs, std::vector<size_t>* offsets = nullptr) {
  size_t body = 0;
  for (auto& m : msgs) {
    m.data.pad8();
    body += 8 + m.data.size();
  }
  Bytes h;
  h.u8(1);
  h.u8(0);
  h.u16((unsigned)msgs.size());
  h.u32(1);  // reference count
  h.u32((uint32_t)body);
  h.zeros(4);  // messages start 8-byte aligned
  for (auto& m : msgs) {
    h.u16(m.type);
    h.u16((unsigned)m.data.size());
    h.u8(m.flags);
    h.zeros(3);
    if (offsets) offsets->push_back(h.size());
    h.raw(m.data.b.data(), m.data.size());
  }
  return h;
}

// ---- the file -----------------------------------------------------------

struct Entry {
  std::string name;
  uint64_t header;             // object header address
  bool group;
  uint64_t btree, heap;        // groups: their symbol table
};

// Where the pieces of a symbol table go: appended at the end of the file, or
// into [at, end) of a reserved region.
struct Sink {
  bool append;
  uint64_t at, end;
};

// The root table's reserved region for `cap` entries: name heap (header +
// data segment of kHeapPerEntry bytes per entry, the "" at offset 0 and room
// for a free block), then room for the most nodes and B-tree nodes `cap`
// entries take.
constexpr uint64_t kHeapPerEntry = 16;  // a name of up to 15 characters, NUL, 8-byte aligned
uint64_t HeapData(uint64_t cap) { return 8 + kHeapPerEntry * cap + 16; }
uint64_t RegionBytes(uint64_t cap) {
  uint64_t nodes = std::max<uint64_t>(1, (cap + 2 * kLeafK - 1) / (2 * kLeafK));
  uint64_t bytes = 32 + HeapData(cap) + nodes * kSnodBytes;
  for (;;) {  // B-tree levels
    nodes = (nodes + 2 * kNodeK - 1) / (2 * kNodeK);
    bytes += nodes * kTreeBytes;
    if (nodes == 1) return bytes;
  }
}

class H5File {
 public:
  ~H5File() {
    if (f_) std::fclose(f_);
  }
  bool Create(const char* path) {
    f_ = std::fopen(path, "w+b");
    eof_ = kSuperblockBytes;
    return f_ != nullptr;
  }
  bool Open(const char* path) {
    f_ = std::fopen(path, "r+b");
    if (!f_) return false;
    uint8_t sb[kSuperblockBytes];
    if (!ReadAt(0, sb, sizeof(sb)) || std::memcmp(sb, "\x89HDF\r\n\x1a\n", 8) != 0 || sb[8] != 0 || sb[13] != 8 ||
        sb[14] != 8 || Rd64(sb + 24) != 0)
      return false;
    eof_ = Rd64(sb + 40);
    root_header_ = Rd64(sb + kRootEntryAt + 8);
    // the root group's symbol-table message, rewritten by each save
    uint8_t oh[16];
    if (!ReadAt(root_header_, oh, sizeof(oh)) || oh[0] != 1) return false;
    const unsigned n = Rd16(oh + 2);
    uint64_t at = root_header_ + 16;
    for (unsigned i = 0; i < n; ++i) {
      uint8_t mh[8];
      if (!ReadAt(at, mh, sizeof(mh))) return false;
      if (Rd16(mh) == MSG_SYMBOL_TABLE) root_stab_ = at + 8;
      at += 8 + Rd16(mh + 2);
    }
    uint8_t st[16];
    if (!root_stab_ || !ReadAt(root_stab_, st, sizeof(st))) return false;
    // the root table's region: its heap starts it; the heap's data size gives
    // the capacity (a heap without a free block belongs to no region)
    uint8_t hh[32];
    const uint64_t heap = Rd64(st + 8);
    if (!ReadAt(heap, hh, sizeof(hh))) return false;
    const uint64_t data = Rd64(hh + 8), cap = data >= 24 ? (data - 24) / kHeapPerEntry : 0;
    if (Rd64(hh + 16) != kHeapFreeNull && Rd64(hh + 24) == heap + 32 && HeapData(cap) == data &&
        heap + RegionBytes(cap) <= eof_) {
      region_at_ = heap;
      region_cap_ = cap;
    }
    return ReadGroup(Rd64(st), heap, &root_);
  }

  uint64_t Append(const void* p, size_t n) {
    const uint64_t at = eof_;
    if (!WriteAt(at, p, n)) return kUndef;
    eof_ += (n + 7) & ~size_t(7);
    return at;
  }
  uint64_t Append(const Bytes& b) { return Append(b.b.data(), b.size()); }

  // A contiguous float64 dataset; returns its object header address.
  uint64_t Dataset(const std::vector<uint64_t>& dims, const double* data) {
    uint64_t n = 1;
    for (uint64_t d : dims) n *= d;
    const uint64_t raw = Append(data, n * sizeof(double));
    std::vector<Msg> msgs;
    msgs.push_back({MSG_DATASPACE, 0, DataspaceBody(dims)});
    msgs.push_back({MSG_DATATYPE, 1, DoubleType()});
    Msg fill{MSG_FILL, 1, {}};  // version 1: allocation late, write if set, default value
    fill.data.u8(1);
    fill.data.u8(2);
    fill.data.u8(2);
    fill.data.u8(1);
    fill.data.u32(0);
    msgs.push_back(fill);
    Msg layout{MSG_LAYOUT, 0, {}};  // version 3, contiguous
    layout.data.u8(3);
    layout.data.u8(1);
    layout.data.u64(raw);
    layout.data.u64(n * sizeof(double));
    msgs.push_back(layout);
    if (raw == kUndef) return kUndef;
    return Append(ObjectHeader(msgs));
  }

  // Writes b at the sink's next position; *where receives its address.
  bool Put(Sink& sink, const Bytes& b, uint64_t* where) {
    if (sink.append) {
      *where = Append(b);
      return *where != kUndef;
    }
    const uint64_t n = (b.size() + 7) & ~uint64_t(7);
    if (sink.at + n > sink.end || !WriteAt(sink.at, b.b.data(), b.size())) return false;
    *where = sink.at;
    sink.at += n;
    return true;
  }

  // The symbol table of a group with these members: name heap, nodes and
  // B-tree; *btree and *heap receive their addresses.  heap_data: the size
  // of the heap's data segment (0: just the names; larger: the rest is one
  // free block of at least 16 bytes).  False when the table does not fit.
  bool SymbolTableOf(std::vector<Entry> members, uint64_t* btree, uint64_t* heap) {
    Sink sink{true, 0, 0};
    return SymbolTableOf(std::move(members), btree, heap, sink, 0);
  }
  bool SymbolTableOf(std::vector<Entry> members, uint64_t* btree, uint64_t* heap, Sink& sink, uint64_t heap_data) {
    std::sort(members.begin(), members.end(), [](const Entry& a, const Entry& b) {
      return std::strcmp(a.name.c_str(), b.name.c_str()) < 0;
    });
    // local heap: "" at offset 0, then each name, NUL-terminated, 8-byte aligned
    Bytes names;
    names.zeros(8);
    std::vector<uint64_t> off;
    for (const auto& e : members) {
      off.push_back(names.size());
      names.raw(e.name.c_str(), e.name.size() + 1);
      names.pad8();
    }
    const uint64_t used = names.size();
    if (heap_data != 0) {  // the unused tail as one free block: next (none), size
      if (used + 16 > heap_data) return false;
      names.u64(kHeapFreeNull);
      names.u64(heap_data - used);
      names.zeros(heap_data - used - 16);
    }
    Bytes h;
    h.raw("HEAP", 4);
    h.u8(0);
    h.zeros(3);
    h.u64(names.size());
    h.u64(heap_data != 0 ? used : kHeapFreeNull);
    const uint64_t heap_at = sink.append ? eof_ : sink.at;
    h.u64(heap_at + 32);  // data segment right after the header
    h.raw(names.b.data(), names.size());
    uint64_t at_h;
    if (!Put(sink, h, &at_h) || at_h != heap_at) return false;
    // symbol-table nodes of up to 2K entries, filled evenly
    const size_t n = members.size();
    const size_t nodes = std::max<size_t>(1, (n + 2 * kLeafK - 1) / (2 * kLeafK));
    std::vector<uint64_t> child, key;  // key[i]: heap offset of the largest name under child i
    size_t first = 0;
    for (size_t s = 0; s < nodes; ++s) {
      const size_t last = n * (s + 1) / nodes;
      Bytes node;
      node.raw("SNOD", 4);
      node.u8(1);
      node.u8(0);
      node.u16((unsigned)(last - first));
      for (size_t i = first; i < last; ++i) {
        const Entry& e = members[i];
        node.u64(off[i]);
        node.u64(e.header);
        node.u32(e.group ? 1 : 0);
        node.u32(0);
        if (e.group) {
          node.u64(e.btree);
          node.u64(e.heap);
        } else {
          node.zeros(16);
        }
      }
      node.zeros(kSnodBytes - node.size());
      uint64_t at;
      if (!Put(sink, node, &at)) return false;
      child.push_back(at);
      key.push_back(last > first ? off[last - 1] : 0);
      first = last;
    }
    // B-tree levels: up to 2K children per node, siblings linked
    uint64_t left_key = 0;  // the key left of the first child of a level: ""
    for (int level = 0;; ++level) {
      const size_t m = child.size();
      const size_t groups = (m + 2 * kNodeK - 1) / (2 * kNodeK);
      std::vector<uint64_t> addr(groups);
      const uint64_t base = sink.append ? eof_ : sink.at;
      for (size_t g = 0; g < groups; ++g) addr[g] = base + g * (uint64_t)kTreeBytes;
      std::vector<uint64_t> up_child, up_key;
      size_t c0 = 0;
      for (size_t g = 0; g < groups; ++g) {
        const size_t c1 = m * (g + 1) / groups;
        Bytes t;
        t.raw("TREE", 4);
        t.u8(0);  // group node
        t.u8((unsigned)level);
        t.u16((unsigned)(c1 - c0));
        t.u64(g > 0 ? addr[g - 1] : kUndef);
        t.u64(g + 1 < groups ? addr[g + 1] : kUndef);
        t.u64(c0 == 0 ? left_key : key[c0 - 1]);
        for (size_t c = c0; c < c1; ++c) {
          t.u64(child[c]);
          t.u64(key[c]);
        }
        t.zeros(kTreeBytes - t.size());
        uint64_t at_t;
        if (!Put(sink, t, &at_t) || at_t != addr[g]) return false;
        up_child.push_back(addr[g]);
        up_key.push_back(key[c1 - 1]);
        c0 = c1;
      }
      if (groups == 1) {
        *btree = addr[0];
        break;
      }
      child.swap(up_child);
      key.swap(up_key);
    }
    *heap = heap_at;
    return true;
  }

  // Writes the superblock, with the root group at root_header_.
  bool Superblock(uint64_t root_btree, uint64_t root_heap) {
    Bytes s;
    s.raw("\x89HDF\r\n\x1a\n", 8);
    s.u8(0);  // superblock version
    s.u8(0);  // free-space storage version
    s.u8(0);  // root group symbol-table entry version
    s.u8(0);
    s.u8(0);  // shared header message format version
    s.u8(8);  // size of offsets
    s.u8(8);  // size of lengths
    s.u8(0);
    s.u16(kLeafK);
    s.u16(kNodeK);
    s.u32(0);  // consistency flags
    s.u64(0);  // base address
    s.u64(kUndef);  // free-space info
    s.u64(eof_);
    s.u64(kUndef);  // driver information block
    s.u64(0);  // root entry: name offset ""
    s.u64(root_header_);
    s.u32(1);  // cached symbol table
    s.u32(0);
    s.u64(root_btree);
    s.u64(root_heap);
    return WriteAt(0, s.b.data(), s.size());
  }

  // The root table into its region (a new one, twice the entries, when it
  // does not fit the current one).
  bool RootTable(uint64_t* bt, uint64_t* hp) {
    if (region_cap_ < root_.size() || !TryRegion(bt, hp)) {
      region_cap_ = std::max<uint64_t>(64, 2 * root_.size());
      const uint64_t bytes = RegionBytes(region_cap_);
      const std::vector<uint8_t> zero(bytes, 0);
      region_at_ = Append(zero.data(), zero.size());
      if (region_at_ == kUndef) return false;
      return TryRegion(bt, hp);
    }
    return true;
  }
  bool TryRegion(uint64_t* bt, uint64_t* hp) {
    Sink sink{false, region_at_, region_at_ + RegionBytes(region_cap_)};
    return SymbolTableOf(root_, bt, hp, sink, HeapData(region_cap_));
  }

  bool WriteRoot(const std::vector<Msg>& attrs) {
    uint64_t bt, hp;
    if (!RootTable(&bt, &hp)) return false;
    std::vector<Msg> msgs{SymbolTable(bt, hp)};
    msgs.insert(msgs.end(), attrs.begin(), attrs.end());
    std::vector<size_t> at;
    root_header_ = Append(ObjectHeader(msgs, &at));
    if (root_header_ == kUndef) return false;
    root_stab_ = root_header_ + at[0];
    return Superblock(bt, hp);
  }

  // Points the root group at a new symbol table holding root_.
  bool UpdateRoot() {
    uint64_t bt, hp;
    if (!RootTable(&bt, &hp)) return false;
    Bytes st;
    st.u64(bt);
    st.u64(hp);
    return WriteAt(root_stab_, st.b.data(), st.size()) && Superblock(bt, hp);
  }

  std::vector<Entry> root_;

 private:
  bool WriteAt(uint64_t at, const void* p, size_t n) {
    return std::fseek(f_, (long)at, SEEK_SET) == 0 && std::fwrite(p, 1, n, f_) == n;
  }
  bool ReadAt(uint64_t at, void* p, size_t n) {
    return std::fseek(f_, (long)at, SEEK_SET) == 0 && std::fread(p, 1, n, f_) == n;
  }
  // Members of a group this writer made: walks the B-tree down to its nodes.
  bool ReadGroup(uint64_t btree, uint64_t heap, std::vector<Entry>* out) {
    uint8_t hh[32];
    if (!ReadAt(heap, hh, sizeof(hh)) || std::memcmp(hh, "HEAP", 4) != 0) return false;
    std::vector<uint8_t> names(Rd64(hh + 8));
    if (!ReadAt(Rd64(hh + 24), names.data(), names.size())) return false;
    return ReadNode(btree, names, out);
  }
  bool ReadNode(uint64_t at, const std::vector<uint8_t>& names, std::vector<Entry>* out) {
    std::vector<uint8_t> t(kTreeBytes);
    if (!ReadAt(at, t.data(), t.size()) || std::memcmp(t.data(), "TREE", 4) != 0) return false;
    const int level = t[5];
    const unsigned used = Rd16(&t[6]);
    for (unsigned c = 0; c < used; ++c) {
      const uint64_t child = Rd64(&t[24 + 8 + 16 * c]);
      if (level > 0) {
        if (!ReadNode(child, names, out)) return false;
        continue;
      }
      std::vector<uint8_t> s(kSnodBytes);
      if (!ReadAt(child, s.data(), s.size()) || std::memcmp(s.data(), "SNOD", 4) != 0) return false;
      const unsigned k = Rd16(&s[6]);
      for (unsigned i = 0; i < k; ++i) {
        const uint8_t* e = &s[8 + kEntryBytes * i];
        const uint64_t off = Rd64(e);
        if (off >= names.size()) return false;
        Entry en;
        en.name.assign((const char*)&names[off], strnlen((const char*)&names[off], names.size() - off));
        en.header = Rd64(e + 8);
        en.group = Rd64(e + 16) == 1;
        en.btree = Rd64(e + 24);
        en.heap = Rd64(e + 32);
        out->push_back(en);
      }
    }
    return true;
  }

  FILE* f_ = nullptr;
  uint64_t eof_ = 0;
  uint64_t root_header_ = 0, root_stab_ = 0;
  uint64_t region_at_ = 0, region_cap_ = 0;  // the root table's reserved region
};

}  // namespace

extern "C" int fv_h5_save(const fv_params* p, const char* path, int iteration, double t, const double* rho,
                          const double* u, const double* v, const double* w, const double* prs) {
  if (!p || !path || iteration < 0 || !rho || !u || !v || !w || !prs) return FV_ERR_PARAM;
  const int nx = p->Nx, ny = p->Ny, nz = p->Nz, ng = p->Ng;
  if (nx < 1 || ny < 1 || nz < 1) return FV_ERR_PARAM;
  H5File f;
  std::vector<Msg> root_attrs;
  if (iteration == 0) {
    if (!f.Create(path)) return FV_ERR_IO;
    // vertex coordinates as IOManager.h:115-124 builds them
    const size_t nv = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    std::vector<double> xyz[3];
    for (auto& a : xyz) a.reserve(nv);
    for (int k = 0; k <= nz; ++k)
      for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
          xyz[0].push_back(i * p->dx);
          xyz[1].push_back(j * p->dy);
          xyz[2].push_back(k * p->dz);
        }
    for (int a = 0; a < 3; ++a) {
      const uint64_t h = f.Dataset({nv}, xyz[a].data());
      if (h == kUndef) return FV_ERR_IO;
      f.root_.push_back({std::string(1, "xyz"[a]), h, false, 0, 0});
    }
    const struct {
      const char* name;
      int value;
    } ints[] = {{"Ntx", nx + 2 * ng}, {"Nty", ny + 2 * ng}, {"Ntz", nz + 2 * ng}, {"Nx", nx}, {"Ny", ny},
                {"Nz", nz}, {"ibeg", ng}, {"iend", ng + nx}, {"jbeg", ng}, {"jend", ng + ny}, {"kbeg", ng},
                {"kend", ng + nz}};
    for (const auto& a : ints) {
      const int32_t val = a.value;
      root_attrs.push_back(Attribute(a.name, Int32Type(), &val, sizeof(val)));
    }
    const std::string prob(p->problem, strnlen(p->problem, sizeof(p->problem)));
    root_attrs.push_back(Attribute("problem", StringType((uint32_t)prob.size() + 1), prob.c_str(), prob.size() + 1));
  } else if (!f.Open(path)) {
    return FV_ERR_IO;
  }
  // the group ite_<iteration>: five [Nz][Ny][Nx] fields and the time
  const std::vector<uint64_t> dims{(uint64_t)nz, (uint64_t)ny, (uint64_t)nx};
  const double* fields[5] = {rho, u, v, w, prs};
  const char* names[5] = {"rho", "u", "v", "w", "prs"};
  std::vector<Entry> members;
  for (int k = 0; k < 5; ++k) {
    const uint64_t h = f.Dataset(dims, fields[k]);
    if (h == kUndef) return FV_ERR_IO;
    members.push_back({names[k], h, false, 0, 0});
  }
  uint64_t bt, hp;
  if (!f.SymbolTableOf(members, &bt, &hp)) return FV_ERR_IO;
  const uint64_t gh = f.Append(ObjectHeader({SymbolTable(bt, hp), Attribute("time", DoubleType(), &t, sizeof(t))}));
  if (gh == kUndef) return FV_ERR_IO;
  const std::string gname = "ite_" + std::to_string(iteration);
  f.root_.erase(std::remove_if(f.root_.begin(), f.root_.end(), [&](const Entry& e) { return e.name == gname; }),
                f.root_.end());
  f.root_.push_back({gname, gh, true, bt, hp});
  if (iteration == 0) return f.WriteRoot(root_attrs) ? FV_OK : FV_ERR_IO;
  return f.UpdateRoot() ? FV_OK : FV_ERR_IO;
}
