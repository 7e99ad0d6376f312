// mat73.cpp -- MATLAB -v7.3 MAT-files on the host: the part of HDF5 that
// MATLAB's save -v7.3 writes, read without the HDF5 library.
//
// No counterpart in the reference (its data files are read in MATLAB).  A
// -v7.3 MAT-file is an HDF5 file behind a 512-byte user block holding
// MATLAB's text header; MATLAB needs this format for any array above 2 GB, so
// full-size scans come in it.  Each variable is an object of the root group:
// a numeric array is a dataset with a MATLAB_class attribute and the MATLAB
// dimensions reversed (HDF5 is row-major, MATLAB column-major: the bytes are
// already in MATLAB's order); a complex array is a compound {real, imag};
// structs, cells and sparse arrays are groups.  Read here, written from the
// HDF5 file format specification (version 3.0):
//  - superblocks of versions 0-3; object headers of versions 1 and 2 with
//    their continuation blocks;
//  - groups held in a symbol table (version 1 B-tree of group nodes, symbol
//    table nodes, local heap) or in link messages; dense groups (fractal
//    heap) are refused;
//  - datasets: dataspace messages v1/v2; fixed-point and IEEE floating-point
//    types in either byte order and compounds (their first member: MATLAB's
//    real part); compact, contiguous and chunked layouts (layout message v3
//    with a version 1 B-tree of chunks, v4 with a single-chunk index);
//    the deflate, shuffle and Fletcher-32 filters (the checksum is dropped,
//    not verified);
//  - attributes v1-v3, for MATLAB_class and MATLAB_empty.
// A chunked dataset's chunks are decoded on several host threads.
// Written (mat73_write): single-precision variables as MATLAB lays them out
// (version 0 superblock, version 1 object headers, a symbol-table root group,
// contiguous data with MATLAB_class "single"); appending relinks the root
// group at the end of the file.
// Every offset is checked against the file size, every walk is bounded: a
// damaged file gives an error, not a crash.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "fileio_internal.h"

namespace mexct {
mexct_status set_err(mexct_status code, const char* fmt, ...);
}

namespace {

using mexct::Mat73Var;
using mexct::set_err;

// A structure the reader cannot follow: malformed (I/O error) or valid HDF5
// outside what is read here (unsupported).
struct Bad {
  const char* what;
  bool unsupported;
};
[[noreturn]] void bad(const char* what) { throw Bad{what, false}; }
[[noreturn]] void unsupported(const char* what) { throw Bad{what, true}; }

const uint8_t kSignature[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

// The file's bytes with checked little-endian reads, and the superblock's
// sizes of offsets and lengths and base address (addresses are relative to
// the superblock's position, after any user block).
class File {
 public:
  explicit File(const std::vector<uint8_t>& f) : p_(f.data()), n_(f.size()) {}
  File(const uint8_t* p, uint64_t n) : p_(p), n_(n) {}
  uint64_t size() const { return n_; }
  const uint8_t* at(uint64_t off, uint64_t len) const {
    if (off > n_ || len > n_ - off) bad("a structure runs past the end of the file");
    return p_ + off;
  }
  uint64_t uint(uint64_t off, int bytes) const {
    const uint8_t* q = at(off, (uint64_t)bytes);
    uint64_t v = 0;
    for (int i = bytes - 1; i >= 0; --i) v = (v << 8) | q[i];
    return v;
  }
  uint32_t u8(uint64_t off) const { return *at(off, 1); }
  uint32_t u16(uint64_t off) const { return (uint32_t)uint(off, 2); }
  uint32_t u32(uint64_t off) const { return (uint32_t)uint(off, 4); }
  bool sig4(uint64_t off, const char* s) const {
    return off <= n_ && n_ - off >= 4 && std::memcmp(p_ + off, s, 4) == 0;
  }
  uint64_t len(uint64_t off) const { return uint(off, sl); }
  bool defined(uint64_t off) const {
    const uint64_t a = uint(off, so);
    return so >= 8 ? a != ~0ull : a != (1ull << (8 * so)) - 1;
  }
  // The address stored at off, as a file offset.
  uint64_t addr(uint64_t off) const {
    if (!defined(off)) bad("an undefined address where an object is expected");
    const uint64_t a = uint(off, so);
    if (base > n_ || a >= n_ - base) bad("an address beyond the end of the file");
    return base + a;
  }

  int so = 8, sl = 8;
  uint64_t base = 0;
  uint64_t visits = 0;  // B-tree nodes and header blocks walked (bounded)

 private:
  const uint8_t* p_;
  uint64_t n_;
};

void visit(File& h) {
  if (++h.visits > (1u << 22)) bad("too many B-tree nodes or header blocks");
}

// ---- superblock -------------------------------------------------------------

struct Root {
  uint64_t header = 0;           // the root group's object header
  bool cached = false;           // a symbol table in the superblock's root entry
  uint64_t btree = 0, heap = 0;
};

bool find_superblock(const File& h, uint64_t* off) {
  for (uint64_t o = 0; o <= h.size() && h.size() - o >= 8; o = o == 0 ? 512 : 2 * o)
    if (std::memcmp(h.at(o, 8), kSignature, 8) == 0) {
      *off = o;
      return true;
    }
  return false;
}

Root superblock(File& h) {
  uint64_t s = 0;
  if (!find_superblock(h, &s)) bad("no HDF5 superblock");
  const uint32_t ver = h.u8(s + 8);
  Root r;
  auto sizes = [&](uint32_t so, uint32_t sl) {
    if ((so != 2 && so != 4 && so != 8) || (sl != 2 && sl != 4 && sl != 8))
      bad("sizes of offsets / lengths other than 2, 4 or 8");
    h.so = (int)so;
    h.sl = (int)sl;
    h.base = s;  // what the HDF5 library does: addresses count from the superblock
  };
  if (ver <= 1) {
    sizes(h.u8(s + 13), h.u8(s + 14));
    // base, free-space, end-of-file and driver addresses, then the root entry
    const uint64_t e = s + (ver == 1 ? 28 : 24) + 4 * (uint64_t)h.so;
    r.header = h.addr(e + h.so);
    if (h.u32(e + 2 * h.so) == 1) {  // cache type 1: B-tree and local heap
      r.cached = true;
      r.btree = h.addr(e + 2 * h.so + 8);
      r.heap = h.addr(e + 3 * h.so + 8);
    }
  } else if (ver == 2 || ver == 3) {
    sizes(h.u8(s + 9), h.u8(s + 10));
    r.header = h.addr(s + 12 + 3 * (uint64_t)h.so);  // after base, extension, end of file
  } else {
    unsupported("a superblock version above 3");
  }
  return r;
}

// ---- object headers ---------------------------------------------------------

struct Msg {
  uint32_t type;
  uint64_t off, size;
};

std::vector<Msg> messages(File& h, uint64_t oh) {
  std::vector<Msg> out;
  std::vector<std::pair<uint64_t, uint64_t>> blocks;  // message areas [begin, end)
  const bool v2 = h.sig4(oh, "OHDR");
  uint32_t flags = 0;
  if (v2) {
    if (h.u8(oh + 4) != 2) unsupported("an object header version other than 1 or 2");
    flags = h.u8(oh + 5);
    uint64_t q = oh + 6 + ((flags & 0x20) ? 16 : 0) + ((flags & 0x10) ? 4 : 0);
    const int cs = 1 << (flags & 3);
    const uint64_t size0 = h.uint(q, cs);
    q += cs;
    h.at(q, size0);
    blocks.push_back({q, q + size0});
  } else {
    if (h.u8(oh) != 1) bad("not an object header");
    const uint64_t size0 = h.u32(oh + 8);
    h.at(oh + 16, size0);
    blocks.push_back({oh + 16, oh + 16 + size0});
  }
  // message header: type, size, flags (+ creation order) / type, size, flags, reserved
  const uint64_t mh = v2 ? 4 + ((flags & 0x04) ? 2 : 0) : 8;
  for (size_t b = 0; b < blocks.size(); ++b) {
    visit(h);
    uint64_t q = blocks[b].first;
    const uint64_t end = blocks[b].second;
    while (end - q >= mh) {
      const uint32_t type = v2 ? h.u8(q) : h.u16(q);
      const uint64_t size = v2 ? h.u16(q + 1) : h.u16(q + 2);
      const uint64_t d = q + mh;
      if (size > end - d) bad("an object header message runs past its block");
      if (type == 0x10) {  // continuation: address, length
        const uint64_t a = h.addr(d), l = h.len(d + h.so);
        h.at(a, l);
        if (v2) {
          if (l < 8 || !h.sig4(a, "OCHK")) bad("a bad object header continuation block");
          blocks.push_back({a + 4, a + l - 4});
        } else {
          blocks.push_back({a, a + l});
        }
      } else if (type != 0) {
        out.push_back({type, d, size});
      }
      q = d + size;
    }
  }
  return out;
}

// ---- datatypes, dataspaces, layouts, filters, attributes -------------------

struct Type {
  int cls = -1;      // 0 fixed-point, 1 IEEE floating-point
  uint32_t size = 0;  // bytes of one element
  bool be = false, sgn = false;
  uint32_t esize = 0, moff = 0;  // the converted value: bytes and offset in the element
};

Type datatype(const File& h, uint64_t off, uint64_t end, int depth = 0) {
  if (depth > 8) bad("nested compound types");
  Type t;
  const uint32_t b0 = h.u8(off), cls = b0 & 0x0f, ver = b0 >> 4;
  const uint32_t f0 = h.u8(off + 1), f1 = h.u8(off + 2);
  t.size = h.u32(off + 4);
  if (cls == 0 || cls == 1) {
    t.cls = (int)cls;
    t.be = f0 & 1;
    t.sgn = cls == 0 && (f0 & 0x08);
    if (cls == 1 && (f0 & 0x40)) unsupported("VAX floating-point byte order");
    const bool ok = cls == 0 ? (t.size == 1 || t.size == 2 || t.size == 4 || t.size == 8)
                             : (t.size == 4 || t.size == 8);
    if (!ok) unsupported("a numeric type of an unusual size");
    t.esize = t.size;
    return t;
  }
  if (cls == 6) {  // compound: its first member (MATLAB complex arrays: real, imag)
    if ((f0 | (f1 << 8)) < 1) bad("a compound type without members");
    uint64_t q = off + 8;
    uint64_t nl = 0;
    while (h.u8(q + nl) != 0) {
      if (q + nl + 1 >= end) bad("a compound member name runs past its message");
      ++nl;
    }
    uint64_t moff;
    if (ver < 3) {
      q += (nl + 1 + 7) / 8 * 8;
      moff = h.u32(q);
      q += 4;
      if (ver == 1) q += 28;  // dimensionality, reserved, permutation, reserved, sizes
    } else {
      q += nl + 1;
      int ob = 1;  // bytes of the member offset: the fewest that hold the type's size
      while (ob < 4 && (1ull << (8 * ob)) <= t.size) ++ob;
      moff = h.uint(q, ob);
      q += ob;
    }
    const Type m = datatype(h, q, end, depth + 1);
    t.cls = m.cls;
    t.be = m.be;
    t.sgn = m.sgn;
    t.esize = m.esize;
    t.moff = (uint32_t)moff + m.moff;
    if ((uint64_t)t.moff + t.esize > t.size) bad("a compound member outside its element");
    return t;
  }
  unsupported("a datatype that is neither numeric nor a compound of numbers");
}

std::vector<uint64_t> dataspace(const File& h, uint64_t off, bool* null_space) {
  const uint32_t ver = h.u8(off), rank = h.u8(off + 1);
  uint64_t q;
  *null_space = false;
  if (ver == 1) {
    q = off + 8;
  } else if (ver == 2) {
    q = off + 4;
    *null_space = h.u8(off + 3) == 2;
  } else {
    unsupported("a dataspace message version other than 1 or 2");
  }
  if (rank > 32) bad("a dataspace of more than 32 dimensions");
  std::vector<uint64_t> d(rank);
  for (uint32_t i = 0; i < rank; ++i) d[i] = h.len(q + (uint64_t)i * h.sl);
  return d;
}

struct Layout {
  int cls = -1;                 // 0 compact, 1 contiguous, 2 chunked
  bool stored = false;          // data written (an undefined address reads as zeros)
  uint64_t data = 0, size = 0;  // compact / contiguous bytes; single chunk
  uint64_t btree = 0;           // chunked: B-tree of chunks
  bool single = false;          // chunked, v4: one chunk
  uint32_t single_mask = 0;
  std::vector<uint64_t> chunk;  // chunk dimensions (the dataset's rank)
};

Layout layout(const File& h, uint64_t off, uint64_t end, size_t rank, uint32_t esz) {
  Layout L;
  const uint32_t ver = h.u8(off);
  if (ver != 3 && ver != 4) unsupported("a data layout message version other than 3 or 4");
  L.cls = (int)h.u8(off + 1);
  if (L.cls == 0) {
    L.size = h.u16(off + 2);
    L.data = off + 4;
    if (L.size > end - L.data) bad("compact data past its message");
    L.stored = true;
  } else if (L.cls == 1) {
    L.stored = h.defined(off + 2);
    if (L.stored) L.data = h.addr(off + 2);
    L.size = h.len(off + 2 + h.so);
  } else if (L.cls == 2) {
    uint32_t nd;
    uint64_t q;
    int enc = 4;
    if (ver == 3) {
      nd = h.u8(off + 2);
      L.stored = h.defined(off + 3);
      if (L.stored) L.btree = h.addr(off + 3);
      q = off + 3 + h.so;
    } else {
      nd = h.u8(off + 3);
      enc = (int)h.u8(off + 4);
      if (enc < 1 || enc > 8) bad("a chunk dimension encoding of more than 8 bytes");
      q = off + 5;
    }
    if (nd != rank + 1) bad("chunk dimensions that do not match the dataspace");
    for (uint32_t i = 0; i < nd; ++i) {
      const uint64_t c = h.uint(q + (uint64_t)i * enc, enc);
      if (i + 1 < nd) {
        if (c == 0) bad("a zero chunk dimension");
        L.chunk.push_back(c);
      } else if (c != esz) {
        bad("a chunk element size that is not the datatype's");
      }
    }
    q += (uint64_t)nd * enc;
    if (ver == 4) {
      const uint32_t flags = h.u8(off + 2), index = h.u8(q);
      if (index != 1) unsupported("a chunk index other than a B-tree or a single chunk");
      L.single = true;
      ++q;
      if (flags & 0x02) {  // filtered single chunk: its size and filter mask
        L.size = h.len(q);
        L.single_mask = h.u32(q + h.sl);
        q += h.sl + 4;
      } else {
        uint64_t n = esz;
        for (uint64_t c : L.chunk) n *= c;
        L.size = n;
      }
      L.stored = h.defined(q);
      if (L.stored) L.data = h.addr(q);
    }
  } else {
    unsupported("a virtual or unknown data layout");
  }
  return L;
}

std::vector<uint32_t> filters(const File& h, uint64_t off, uint64_t end) {
  const uint32_t ver = h.u8(off), nf = h.u8(off + 1);
  if (ver != 1 && ver != 2) unsupported("a filter pipeline message version other than 1 or 2");
  std::vector<uint32_t> ids;
  uint64_t q = ver == 1 ? off + 8 : off + 2;
  for (uint32_t i = 0; i < nf; ++i) {
    const uint32_t id = h.u16(q);
    if (ver == 1) {  // id, name length, flags, values, name (padded), values, padding
      const uint64_t name = h.u16(q + 2), nv = h.u16(q + 6);
      q += 8 + name + 4 * nv + ((nv & 1) ? 4 : 0);
    } else {  // id, [name length], flags, values, [name], values
      uint64_t p = q + 2, name = 0;
      if (id >= 256) {
        name = h.u16(p);
        p += 2;
      }
      const uint64_t nv = h.u16(p + 2);
      q = p + 4 + name + 4 * nv;
    }
    if (q > end) bad("a filter pipeline message runs past its end");
    ids.push_back(id);
  }
  return ids;
}

struct Attr {
  std::string name;
  uint64_t type = 0, data = 0;
};

Attr attribute(const File& h, uint64_t off, uint64_t end) {
  const uint32_t ver = h.u8(off);
  if (ver < 1 || ver > 3) unsupported("an attribute message version above 3");
  const uint64_t nsz = h.u16(off + 2), tsz = h.u16(off + 4), ssz = h.u16(off + 6);
  auto pad = [&](uint64_t x) { return ver == 1 ? (x + 7) / 8 * 8 : x; };
  uint64_t q = ver == 3 ? off + 9 : off + 8;
  Attr a;
  const char* s = reinterpret_cast<const char*>(h.at(q, nsz));
  a.name.assign(s, strnlen(s, nsz));
  q += pad(nsz);
  a.type = q;
  q += pad(tsz) + pad(ssz);
  a.data = q;
  if (q > end) bad("an attribute message runs past its end");
  return a;
}

// ---- groups -------------------------------------------------------------------

struct Link {
  std::string name;
  uint64_t header;
};

// A group's local heap: the names of its links.
struct Heap {
  uint64_t data, size;
};

std::string heap_name(const File& h, const Heap& hp, uint64_t o) {
  if (o >= hp.size) bad("a link name outside its local heap");
  const char* s = reinterpret_cast<const char*>(h.at(hp.data + o, hp.size - o));
  const size_t n = strnlen(s, hp.size - o);
  if (n == hp.size - o) bad("an unterminated link name");
  return std::string(s, n);
}

// A symbol table node: entries of link name offset, object header, cache
// type, reserved, scratch pad.
void symbol_node(File& h, const Heap& hp, uint64_t a, std::vector<Link>& out) {
  visit(h);
  if (!h.sig4(a, "SNOD")) bad("a bad symbol table node");
  const uint32_t n = h.u16(a + 6);
  const uint64_t es = 2 * (uint64_t)h.so + 24;
  for (uint32_t i = 0; i < n; ++i) {
    const uint64_t e = a + 8 + i * es;
    out.push_back({heap_name(h, hp, h.uint(e, h.so)), h.addr(e + h.so)});
  }
}

// A version 1 B-tree node of group entries: keys (heap offsets) and children
// (subtrees, or symbol table nodes at level 0).
void group_node(File& h, const Heap& hp, uint64_t a, int depth, std::vector<Link>& out) {
  visit(h);
  if (depth > 32) bad("a group B-tree too deep");
  if (!h.sig4(a, "TREE") || h.u8(a + 4) != 0) bad("a bad group B-tree node");
  const uint32_t level = h.u8(a + 5), used = h.u16(a + 6);
  uint64_t q = a + 8 + 2 * (uint64_t)h.so;
  for (uint32_t i = 0; i < used; ++i) {
    const uint64_t child = h.addr(q + h.sl);
    if (level > 0) group_node(h, hp, child, depth + 1, out);
    else symbol_node(h, hp, child, out);
    q += h.sl + h.so;
  }
}

void symbol_table(File& h, uint64_t btree, uint64_t heap, std::vector<Link>& out) {
  if (!h.sig4(heap, "HEAP")) bad("a bad local heap");
  Heap hp;
  hp.size = h.len(heap + 8);
  hp.data = h.addr(heap + 8 + 2 * (uint64_t)h.sl);
  h.at(hp.data, hp.size);
  group_node(h, hp, btree, 0, out);
}

std::vector<Link> root_links(File& h, const Root& r) {
  std::vector<Link> links;
  bool symtab = false;
  uint64_t bt = 0, hp = 0;
  for (const Msg& m : messages(h, r.header)) {
    const uint64_t end = m.off + m.size;
    if (m.type == 0x11) {  // symbol table: B-tree, local heap
      bt = h.addr(m.off);
      hp = h.addr(m.off + h.so);
      symtab = true;
    } else if (m.type == 0x02) {  // link info: a fractal heap means dense storage
      const uint32_t flags = h.u8(m.off + 1);
      if (h.defined(m.off + 2 + ((flags & 1) ? 8 : 0)))
        unsupported("a dense HDF5 group (more variables than compact storage holds)");
    } else if (m.type == 0x06) {  // link
      if (h.u8(m.off) != 1) unsupported("a link message version other than 1");
      const uint32_t flags = h.u8(m.off + 1);
      uint64_t q = m.off + 2;
      uint32_t ltype = 0;
      if (flags & 0x08) ltype = h.u8(q++);
      if (flags & 0x04) q += 8;
      if (flags & 0x10) q += 1;
      const int ls = 1 << (flags & 3);
      const uint64_t nl = h.uint(q, ls);
      q += ls;
      if (nl > end - q) bad("a link name runs past its message");
      std::string name(reinterpret_cast<const char*>(h.at(q, nl)), nl);
      q += nl;
      if (ltype == 0) links.push_back({name, h.addr(q)});  // soft / external links skipped
    }
  }
  if (!symtab && r.cached) {
    bt = r.btree;
    hp = r.heap;
    symtab = true;
  }
  if (symtab) symbol_table(h, bt, hp, links);
  std::sort(links.begin(), links.end(),
            [](const Link& a, const Link& b) { return a.name < b.name; });
  return links;
}

// ---- datasets -----------------------------------------------------------------

bool numeric_class(const std::string& c) {
  static const char* k[] = {"double", "single", "int8",   "uint8",  "int16",  "uint16",
                            "int32",  "uint32", "int64",  "uint64", "logical"};
  for (const char* x : k)
    if (c == x) return true;
  return false;
}

struct Dataset {
  bool is_dataset = false, have_type = false, have_layout = false, null_space = false;
  bool empty = false;  // MATLAB_empty: the data are the dimensions of an empty array
  std::vector<uint64_t> dims;  // HDF5 order
  Type type;
  Layout lay;
  std::vector<uint32_t> filt;
  std::string mclass;
};

std::string string_value(const File& h, const Attr& a) {
  if ((h.u8(a.type) & 0x0f) != 3) return std::string();
  const uint64_t n = h.u32(a.type + 4);
  const char* s = reinterpret_cast<const char*>(h.at(a.data, n));
  std::string v(s, strnlen(s, n));
  while (!v.empty() && v.back() == ' ') v.pop_back();
  return v;
}

Dataset dataset(File& h, uint64_t header) {
  Dataset D;
  std::vector<Msg> ms = messages(h, header);
  for (const Msg& m : ms)
    if (m.type == 0x01) {
      D.dims = dataspace(h, m.off, &D.null_space);
      D.is_dataset = true;
    }
  for (const Msg& m : ms) {
    const uint64_t end = m.off + m.size;
    if (m.type == 0x03) {
      try {
        D.type = datatype(h, m.off, end);
        D.have_type = true;
      } catch (const Bad& b) {
        if (!b.unsupported) throw;  // a char, reference or string type: not numeric
      }
    } else if (m.type == 0x0B) {
      D.filt = filters(h, m.off, end);
    } else if (m.type == 0x0C) {
      const Attr a = attribute(h, m.off, end);
      if (a.name == "MATLAB_class") {
        D.mclass = string_value(h, a);
      } else if (a.name == "MATLAB_empty" && (h.u8(a.type) & 0x0f) == 0) {
        const uint32_t n = h.u32(a.type + 4);
        if (n >= 1 && n <= 8) D.empty = h.uint(a.data, (int)n) != 0;
      }
    }
  }
  if (D.is_dataset && D.have_type)
    for (const Msg& m : ms)
      if (m.type == 0x08) {
        D.lay = layout(h, m.off, m.off + m.size, D.dims.size(), D.type.size);
        D.have_layout = true;
      }
  return D;
}

float convert(const uint8_t* e, const Type& t) {
  const uint8_t* p = e + t.moff;
  uint8_t b[8];
  for (uint32_t i = 0; i < t.esize; ++i) b[i] = t.be ? p[t.esize - 1 - i] : p[i];
  if (t.cls == 1) {
    if (t.esize == 4) {
      float v;
      std::memcpy(&v, b, 4);
      return v;
    }
    double v;
    std::memcpy(&v, b, 8);
    return (float)v;
  }
  uint64_t u = 0;
  for (int i = (int)t.esize - 1; i >= 0; --i) u = (u << 8) | b[i];
  if (t.sgn && t.esize < 8 && (u >> (8 * t.esize - 1)) & 1) u |= ~0ull << (8 * t.esize);
  return t.sgn ? (float)(int64_t)u : (float)u;
}

// n consecutive elements to float: little-endian float32 / float64 elements
// (the common case on the little-endian hosts this builds for) in bulk, the
// rest one by one.
void convert_run(const uint8_t* src, uint64_t n, const Type& t, float* dst) {
  if (t.cls == 1 && !t.be && t.moff == 0 && t.esize == t.size) {
    if (t.size == 4) {
      std::memcpy(dst, src, n * 4);
      return;
    }
    for (uint64_t i = 0; i < n; ++i) {
      double v;
      std::memcpy(&v, src + 8 * i, 8);
      dst[i] = (float)v;
    }
    return;
  }
  for (uint64_t i = 0; i < n; ++i) dst[i] = convert(src + i * t.size, t);
}

void unshuffle(std::vector<uint8_t>& b, uint32_t es) {
  if (es <= 1) return;
  const size_t n = b.size() / es;
  std::vector<uint8_t> o(b.size());
  for (uint32_t j = 0; j < es; ++j)
    for (size_t i = 0; i < n; ++i) o[i * es + j] = b[j * n + i];
  std::copy(b.begin() + (ptrdiff_t)(n * es), b.end(), o.begin() + (ptrdiff_t)(n * es));
  b.swap(o);
}

void unfilter(const std::vector<uint32_t>& ids, uint32_t mask, uint32_t es,
              std::vector<uint8_t>& b) {
  for (int i = (int)ids.size() - 1; i >= 0; --i) {
    if (i < 32 && ((mask >> i) & 1)) continue;  // filter skipped for this chunk
    if (ids[i] == 1) {
      std::vector<uint8_t> o;
      if (!mexct::zlib_inflate_bytes(b.data(), b.size(), o)) bad("a chunk that does not inflate");
      b.swap(o);
    } else if (ids[i] == 2) {
      unshuffle(b, es);
    } else if (ids[i] == 3) {
      if (b.size() < 4) bad("a chunk shorter than its Fletcher-32 checksum");
      b.resize(b.size() - 4);
    } else {
      unsupported("an HDF5 filter other than deflate, shuffle or Fletcher-32");
    }
  }
}

struct Chunk {
  uint64_t addr, size;
  uint32_t mask;
  std::vector<uint64_t> offset;
};

void chunk_tree(File& h, uint64_t a, size_t rank, int depth, std::vector<Chunk>& out) {
  visit(h);
  if (depth > 32) bad("a chunk B-tree too deep");
  if (!h.sig4(a, "TREE") || h.u8(a + 4) != 1) bad("a bad chunk B-tree node");
  const uint32_t level = h.u8(a + 5), used = h.u16(a + 6);
  const uint64_t ks = 8 + 8 * (uint64_t)(rank + 1);  // size, filter mask, rank + 1 offsets
  uint64_t q = a + 8 + 2 * (uint64_t)h.so;
  for (uint32_t i = 0; i < used; ++i) {
    const uint64_t child = h.addr(q + ks);
    if (level > 0) {
      chunk_tree(h, child, rank, depth + 1, out);
    } else {
      Chunk c{child, h.u32(q), h.u32(q + 4), {}};
      for (size_t d = 0; d < rank; ++d) c.offset.push_back(h.uint(q + 8 + 8 * d, 8));
      out.push_back(std::move(c));
    }
    q += ks + h.so;
  }
}

// Copies a decoded chunk (C elements per dimension, row-major) into the
// dataset (D per dimension, row-major) at offsets o, converting to float.
void place(const uint8_t* data, const std::vector<uint64_t>& D, const std::vector<uint64_t>& C,
           const std::vector<uint64_t>& o, const Type& t, float* out) {
  const size_t r = D.size();
  std::vector<uint64_t> ext(r), idx(r, 0);
  for (size_t d = 0; d < r; ++d) {
    if (o[d] >= D[d] || o[d] % C[d] != 0) bad("a chunk outside its dataset");
    ext[d] = std::min(C[d], D[d] - o[d]);
  }
  for (;;) {
    uint64_t src = 0, dst = 0;
    for (size_t d = 0; d < r; ++d) {
      const uint64_t i = d + 1 < r ? idx[d] : 0;
      src = src * C[d] + i;
      dst = dst * D[d] + o[d] + i;
    }
    convert_run(data + src * t.size, ext[r - 1], t, out + dst);
    int d = (int)r - 2;
    while (d >= 0 && ++idx[d] == ext[d]) idx[d--] = 0;
    if (d < 0) break;
  }
}

uint64_t elements(const std::vector<uint64_t>& dims) {
  uint64_t n = 1;
  for (uint64_t d : dims) {
    if (d != 0 && n > (1ull << 40) / d) bad("a dataset of more than 2^40 elements");
    n *= d;
  }
  return n;
}

// All elements of a numeric dataset as float, in its row-major order.
void read_all(File& h, const Dataset& D, float* out, uint64_t n) {
  const Type& t = D.type;
  const Layout& L = D.lay;
  if (L.cls == 0 || L.cls == 1) {
    if (!L.stored) {
      std::fill(out, out + n, 0.f);
      return;
    }
    if (L.size < n * t.size) bad("a dataset shorter than its dimensions");
    convert_run(h.at(L.data, n * t.size), n, t, out);
    return;
  }
  std::fill(out, out + n, 0.f);  // chunks never written hold the fill value 0
  if (!L.stored || n == 0) return;
  std::vector<Chunk> cs;
  if (L.single) cs.push_back({L.data, L.size, L.single_mask, std::vector<uint64_t>(D.dims.size(), 0)});
  else chunk_tree(h, L.btree, D.dims.size(), 0, cs);
  const uint64_t want = elements(L.chunk) * t.size;
  // Chunks are independent: they are decoded on up to 16 host threads, each
  // writing its own chunks' elements (two chunks at one position, which only
  // a damaged file has, would be two writers of the same elements).
  std::vector<const Chunk*> sorted;
  for (const Chunk& c : cs) sorted.push_back(&c);
  std::sort(sorted.begin(), sorted.end(),
            [](const Chunk* a, const Chunk* b) { return a->offset < b->offset; });
  for (size_t i = 1; i < sorted.size(); ++i)
    if (sorted[i]->offset == sorted[i - 1]->offset) bad("two chunks at one position");
  std::atomic<size_t> next{0};
  std::atomic<bool> failed{false};
  std::mutex mu;
  Bad first{nullptr, false};
  bool oom = false;
  auto work = [&]() {
    std::vector<uint8_t> b;
    try {
      for (size_t i; !failed && (i = next.fetch_add(1)) < cs.size();) {
        const Chunk& c = cs[i];
        const uint8_t* p = h.at(c.addr, c.size);
        b.assign(p, p + c.size);
        unfilter(D.filt, c.mask, t.size, b);
        if (b.size() < want) bad("a chunk shorter than its dimensions");
        if (D.dims.empty()) out[0] = convert(b.data(), t);
        else place(b.data(), D.dims, L.chunk, c.offset, t, out);
      }
    } catch (const Bad& e) {
      std::lock_guard<std::mutex> lk(mu);
      if (!failed.exchange(true)) first = e;
    } catch (const std::bad_alloc&) {
      std::lock_guard<std::mutex> lk(mu);
      oom = true;
      failed = true;
    }
  };
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>(std::min<size_t>(hw, 16), cs.size());
  std::vector<std::thread> pool;
  for (size_t k = 1; k < nt; ++k) {
    try {
      pool.emplace_back(work);
    } catch (const std::system_error&) {
      break;  // fewer threads: the others take their chunks
    }
  }
  work();
  for (std::thread& th : pool) th.join();
  if (oom) throw std::bad_alloc();
  if (failed) throw first;
}

// ---- writing -------------------------------------------------------------------

// Bytes of the metadata written after a variable's data, with the absolute
// file offset of its first byte (addresses are written relative to `base`).
struct Blob {
  std::vector<uint8_t> b;
  uint64_t origin = 0, base = 0;
  uint64_t here() const { return origin + b.size(); }
  uint64_t rel() const { return here() - base; }
  void align8() {
    while (here() % 8) b.push_back(0);
  }
  void u(uint64_t v, int n) {
    for (int i = 0; i < n; ++i) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void raw(const void* p, size_t n) {
    const uint8_t* q = static_cast<const uint8_t*>(p);
    b.insert(b.end(), q, q + n);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
};

constexpr uint64_t kUndef = ~0ull;

// One object header message (version 1 header): type, size, flags, reserved,
// data padded to 8 bytes.
void message(std::vector<uint8_t>& out, uint32_t type, const std::vector<uint8_t>& data) {
  const size_t n = (data.size() + 7) / 8 * 8;
  Blob m;
  m.u(type, 2);
  m.u(n, 2);
  m.u(0, 4);
  m.raw(data.data(), data.size());
  m.zeros(n - data.size());
  out.insert(out.end(), m.b.begin(), m.b.end());
}

void object_header(Blob& out, const std::vector<std::pair<uint32_t, std::vector<uint8_t>>>& msgs) {
  std::vector<uint8_t> body;
  for (const auto& m : msgs) message(body, m.first, m.second);
  out.u(1, 1);  // version
  out.u(0, 1);
  out.u(msgs.size(), 2);
  out.u(1, 4);  // reference count
  out.u(body.size(), 4);
  out.u(0, 4);  // padding to 8 bytes
  out.raw(body.data(), body.size());
}

// MATLAB_class (or another attribute) with a string or a scalar uint8 value.
std::vector<uint8_t> attr_msg(const char* name, const std::string* str, int u8value) {
  Blob a, dt, ds;
  if (str) {
    dt.u(0x13, 1);  // string, version 1; null-terminated ASCII
    dt.u(0, 3);
    dt.u(str->size(), 4);
  } else {
    dt.u(0x10, 1);  // fixed-point, version 1, little-endian unsigned
    dt.u(0, 3);
    dt.u(1, 4);
    dt.u(0, 2);
    dt.u(8, 2);
  }
  ds.u(1, 1);  // scalar dataspace, version 1
  ds.zeros(7);
  const size_t nl = std::strlen(name) + 1;
  a.u(1, 1);
  a.u(0, 1);
  a.u(nl, 2);
  a.u(dt.b.size(), 2);
  a.u(ds.b.size(), 2);
  a.raw(name, nl);
  a.zeros((8 - nl % 8) % 8);
  a.raw(dt.b.data(), dt.b.size());
  a.zeros((8 - dt.b.size() % 8) % 8);
  a.raw(ds.b.data(), ds.b.size());
  if (str) a.raw(str->data(), str->size());
  else a.u((uint64_t)u8value, 1);
  return a.b;
}

// The object header of a single-precision variable whose data sit at `data`
// (relative address), dims in the file's order (MATLAB's reversed).  An empty
// array stores its MATLAB dimensions as uint64 data with MATLAB_empty.
void dataset_header(Blob& out, const std::vector<uint64_t>& fdims, uint64_t data, uint64_t bytes,
                    bool empty) {
  Blob sp, ty, fill, lay;
  sp.u(1, 1);
  sp.u(fdims.size(), 1);
  sp.u(1, 1);  // maximum dimensions present
  sp.zeros(5);
  for (uint64_t d : fdims) sp.u(d, 8);
  for (uint64_t d : fdims) sp.u(d, 8);
  if (empty) {
    ty.u(0x10, 1);  // uint64, little-endian
    ty.u(0, 3);
    ty.u(8, 4);
    ty.u(0, 2);
    ty.u(64, 2);
  } else {
    ty.u(0x11, 1);  // IEEE float32, little-endian
    ty.u(0x20, 1);
    ty.u(31, 1);
    ty.u(0, 1);
    ty.u(4, 4);
    ty.u(0, 2);    // bit offset
    ty.u(32, 2);   // precision
    ty.u(23, 1);   // exponent location
    ty.u(8, 1);    // exponent size
    ty.u(0, 1);    // mantissa location
    ty.u(23, 1);   // mantissa size
    ty.u(127, 4);  // exponent bias
  }
  fill.u(2, 1);  // fill value message v2: allocated early, never written, undefined
  fill.u(1, 1);
  fill.u(2, 1);
  fill.u(0, 1);
  lay.u(3, 1);  // layout v3, contiguous
  lay.u(1, 1);
  lay.u(data, 8);
  lay.u(bytes, 8);
  const std::string single = "single";
  std::vector<std::pair<uint32_t, std::vector<uint8_t>>> msgs = {
      {0x01, sp.b}, {0x03, ty.b}, {0x05, fill.b}, {0x08, lay.b},
      {0x0C, attr_msg("MATLAB_class", &single, 0)}};
  if (empty) msgs.push_back({0x0C, attr_msg("MATLAB_empty", nullptr, 1)});
  object_header(out, msgs);
}

// A root group holding `links` (sorted by name): local heap, symbol table
// nodes of up to 2 leafK entries, one B-tree node of up to 2 intK children,
// and the group's object header.  Returns the relative addresses of the
// header, the B-tree and the heap.
struct RootAddrs {
  uint64_t header, btree, heap;
};

RootAddrs write_root(Blob& out, const std::vector<Link>& links, uint32_t leafK, uint32_t intK) {
  // heap data: "" at 0, then the names, each null-terminated to 8 bytes
  std::vector<uint64_t> name_off;
  Blob heapdata;
  heapdata.zeros(8);
  for (const Link& l : links) {
    name_off.push_back(heapdata.b.size());
    heapdata.raw(l.name.data(), l.name.size());
    heapdata.zeros(8 - l.name.size() % 8);
  }
  out.align8();
  const uint64_t hdata = out.rel();
  out.raw(heapdata.b.data(), heapdata.b.size());
  out.align8();
  const uint64_t heap = out.rel();
  out.raw("HEAP", 4);
  out.u(0, 4);  // version 0, reserved
  out.u(heapdata.b.size(), 8);
  out.u(1, 8);  // no free block: the value the HDF5 library writes and accepts for it
  out.u(hdata, 8);
  // symbol table nodes
  const size_t per = 2 * (size_t)leafK;
  std::vector<uint64_t> snods, last;
  for (size_t i = 0; i < links.size(); i += per) {  // links: at least the new variable
    const size_t n = std::min(per, links.size() - i);
    out.align8();
    snods.push_back(out.rel());
    out.raw("SNOD", 4);
    out.u(1, 1);
    out.u(0, 1);
    out.u(n, 2);
    for (size_t k = 0; k < per; ++k) {
      if (k < n) {
        out.u(name_off[i + k], 8);
        out.u(links[i + k].header, 8);
      } else {
        out.zeros(16);
      }
      out.zeros(24);  // cache type 0, reserved, scratch pad
    }
    last.push_back(name_off[i + n - 1]);
  }
  // one B-tree node (group nodes, level 0), allocated at full size
  out.align8();
  const uint64_t tree = out.rel();
  out.raw("TREE", 4);
  out.u(0, 1);
  out.u(0, 1);
  out.u(snods.size(), 2);
  out.u(kUndef, 8);
  out.u(kUndef, 8);
  out.u(0, 8);  // key 0: the empty name
  for (size_t i = 0; i < 2 * (size_t)intK; ++i) {
    if (i < snods.size()) {
      out.u(snods[i], 8);
      out.u(last[i], 8);
    } else {
      out.zeros(16);
    }
  }
  // the root group's object header: its symbol table
  out.align8();
  const uint64_t header = out.rel();
  Blob st;
  st.u(tree, 8);
  st.u(heap, 8);
  object_header(out, {{0x11, st.b}});
  return {header, tree, heap};
}

bool write_all(FILE* f, const void* p, size_t n) {
  return n == 0 || std::fwrite(p, 1, n, f) == n;
}

// Read-only mapping of a whole file.
struct Mapped {
  const uint8_t* p = nullptr;
  size_t n = 0;
  ~Mapped() {
    if (p) munmap(const_cast<uint8_t*>(p), n);
  }
  bool open(const char* path) {
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) return false;
    struct stat st;
    bool ok = fstat(fd, &st) == 0 && st.st_size > 0;
    if (ok) {
      void* m = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
      ok = m != MAP_FAILED;
      if (ok) {
        p = static_cast<const uint8_t*>(m);
        n = (size_t)st.st_size;
      }
    }
    ::close(fd);
    return ok;
  }
};

Mat73Var describe(File& h, const Link& l) {
  Mat73Var v;
  v.name = l.name;
  v.header = l.header;
  Dataset D;
  try {
    D = dataset(h, l.header);
  } catch (const Bad& b) {
    if (!b.unsupported) throw;
    v.unsupported = b.what;  // listed; reading it reports why (the others stay readable)
    return v;
  }
  v.mclass = D.mclass;
  if (!D.is_dataset) return v;  // a group: struct, cell or sparse array
  v.numeric = D.have_type && D.have_layout && !D.null_space &&
              (D.mclass.empty() || numeric_class(D.mclass));
  if (!v.numeric) return v;
  if (D.empty) {  // the data are the empty array's MATLAB dimensions
    const uint64_t n = elements(D.dims);
    if (n > 8) bad("an empty array of more than 8 dimensions");
    std::vector<float> d(n);
    read_all(h, D, d.data(), n);
    for (float x : d) v.dims.push_back((long long)x);
    while (v.dims.size() < 2) v.dims.push_back(v.dims.empty() ? 0 : 1);
    return v;
  }
  elements(D.dims);  // a damaged dataspace is refused here, not at the caller's allocation
  for (size_t i = D.dims.size(); i-- > 0;) v.dims.push_back((long long)D.dims[i]);
  while (v.dims.size() < 2) v.dims.push_back(1);
  return v;
}

mexct_status fail(const char* path, const Bad& b) {
  return set_err(b.unsupported ? MEXCT_ERR_UNSUPPORTED : MEXCT_ERR_IO,
                 "mat: %s (-v7.3 / HDF5): %s", path, b.what);
}

}  // namespace

namespace mexct {

bool mat73_is_hdf5(const std::vector<uint8_t>& f) {
  uint64_t off;
  return find_superblock(File(f), &off);
}

mexct_status mat73_list(const std::vector<uint8_t>& f, const char* path,
                        std::vector<Mat73Var>& vars) {
  try {
    File h(f);
    const Root r = superblock(h);
    vars.clear();
    for (const Link& l : root_links(h, r)) {
      if (!l.name.empty() && l.name[0] == '#') continue;  // #refs#, #subsystem#
      vars.push_back(describe(h, l));
    }
    return MEXCT_OK;
  } catch (const Bad& b) {
    return fail(path, b);
  } catch (const std::bad_alloc&) {
    return set_err(MEXCT_ERR_OOM, "mat: %s: out of host memory", path);
  }
}

mexct_status mat73_read(const std::vector<uint8_t>& f, const char* path, const Mat73Var& v,
                        float* out, long long count) {
  try {
    File h(f);
    superblock(h);
    const Dataset D = dataset(h, v.header);
    if (!v.numeric || !D.is_dataset || !D.have_type || !D.have_layout)
      return set_err(MEXCT_ERR_UNSUPPORTED, "mat: %s in %s is not a numeric array",
                     v.name.c_str(), path);
    const uint64_t n = D.empty ? 0 : elements(D.dims);
    if ((uint64_t)count != n)
      return set_err(MEXCT_ERR_ARG, "mat: %s holds %llu elements, not %lld", v.name.c_str(),
                     (unsigned long long)n, count);
    if (n == 0) return MEXCT_OK;
    if (!out) return set_err(MEXCT_ERR_ARG, "mat: NULL output");
    read_all(h, D, out, n);
    return MEXCT_OK;
  } catch (const Bad& b) {
    return fail(path, b);
  } catch (const std::bad_alloc&) {
    return set_err(MEXCT_ERR_OOM, "mat: %s: out of host memory", path);
  }
}

mexct_status mat73_write(const char* path, const char* name, const float* data, int ndims,
                         const long long* dims, bool append) {
  const size_t nl = std::strlen(name);
  if (nl == 0 || nl > 63) return set_err(MEXCT_ERR_ARG, "mat: a name of 1 to 63 characters");
  uint64_t n = 1;
  std::vector<uint64_t> fdims;  // the file's order: MATLAB's reversed
  for (int i = ndims - 1; i >= 0; --i) {
    if (dims[i] < 0) return set_err(MEXCT_ERR_ARG, "mat: a negative dimension");
    fdims.push_back((uint64_t)dims[i]);
    if (dims[i] != 0 && n > (1ull << 40) / (uint64_t)dims[i])
      return set_err(MEXCT_ERR_ARG, "mat: more than 2^40 elements");
    n *= (uint64_t)dims[i];
  }
  if (n > 0 && !data) return set_err(MEXCT_ERR_ARG, "mat: NULL data");
  const bool empty = n == 0;
  try {
    std::vector<Link> links;
    uint64_t sb = 512, end = 0;
    int sbver = 0;
    uint32_t leafK = 4, intK = 16;
    if (append) {
      Mapped m;
      if (!m.open(path)) return set_err(MEXCT_ERR_IO, "mat: cannot read %s", path);
      File h(m.p, m.n);
      uint64_t s = 0;
      if (!find_superblock(h, &s)) bad("no HDF5 superblock");
      sbver = (int)h.u8(s + 8);
      if (sbver > 1) unsupported("appending to a file with a version 2 or 3 superblock");
      if (h.u8(s + 13) != 8 || h.u8(s + 14) != 8)
        unsupported("appending to a file whose offsets or lengths are not 8 bytes");
      leafK = h.u16(s + 16);
      intK = h.u16(s + 18);
      if (leafK < 1 || intK < 1) bad("a zero B-tree K in the superblock");
      const Root r = superblock(h);
      links = root_links(h, r);
      for (Link& l : links) {
        if (l.name == name)
          return set_err(MEXCT_ERR_ARG, "mat: %s already holds a variable %s", path, name);
        l.header -= s;  // back to a relative address
      }
      sb = s;
      end = m.n;
    }
    const size_t cap = 2 * (size_t)leafK * 2 * (size_t)intK;
    if (links.size() + 1 > cap)
      unsupported("a root group of more variables than one B-tree node holds");
    FILE* f = std::fopen(path, append ? "r+b" : "wb");
    if (!f) return set_err(MEXCT_ERR_IO, "mat: cannot write %s", path);
    bool ok = true;
    if (!append) {  // MATLAB's user block, then room for the superblock
      char ub[512];
      std::memset(ub, 0, sizeof ub);
      std::memset(ub, ' ', 116);
      const char* txt = "MATLAB 7.3 MAT-file, written by mexct-gb300, HDF5 schema 1.00 .";
      std::memcpy(ub, txt, std::strlen(txt));
      ub[124] = 0x00;  // version 0x0200, little-endian
      ub[125] = 0x02;
      ub[126] = 'I';
      ub[127] = 'M';
      const uint8_t zero[96] = {};
      ok = write_all(f, ub, sizeof ub) && write_all(f, zero, sizeof zero);
      end = 512 + 96;
    } else {
      ok = std::fseek(f, 0, SEEK_END) == 0;
    }
    // the variable's data (8-byte aligned), then its header and the new root
    const uint64_t pad = (8 - end % 8) % 8;
    const uint8_t zeros[8] = {};
    ok = ok && write_all(f, zeros, pad);
    const uint64_t data_at = end + pad;
    uint64_t bytes;
    if (empty) {
      std::vector<uint64_t> md;
      for (int i = 0; i < ndims; ++i) md.push_back((uint64_t)dims[i]);
      bytes = 8 * md.size();
      ok = ok && write_all(f, md.data(), bytes);  // little-endian host
    } else {
      bytes = 4 * n;
      ok = ok && write_all(f, data, bytes);
    }
    Blob meta;
    meta.origin = data_at + bytes;
    meta.base = sb;
    meta.align8();
    const uint64_t vh = meta.rel();
    dataset_header(meta, empty ? std::vector<uint64_t>{(uint64_t)ndims} : fdims, data_at - sb,
                   bytes, empty);
    links.push_back({name, vh});
    std::sort(links.begin(), links.end(),
              [](const Link& a, const Link& b) { return a.name < b.name; });
    const RootAddrs ra = write_root(meta, links, leafK, intK);
    ok = ok && write_all(f, meta.b.data(), meta.b.size());
    const uint64_t eof = meta.here() - sb;
    // superblock: new file, or the changed fields of the old one
    Blob sup;
    if (!append) {
      sup.raw(kSignature, 8);
      sup.u(0, 1);  // superblock, free-space, root entry, reserved, shared header versions
      sup.u(0, 1);
      sup.u(0, 1);
      sup.u(0, 1);
      sup.u(0, 1);
      sup.u(8, 1);  // sizes of offsets and lengths
      sup.u(8, 1);
      sup.u(0, 1);
      sup.u(leafK, 2);
      sup.u(intK, 2);
      sup.u(0, 4);  // consistency flags
      sup.u(0, 8);  // base address
      sup.u(kUndef, 8);
      sup.u(eof, 8);
      sup.u(kUndef, 8);
      sup.u(0, 8);  // root entry: name offset, header, cache type 1, reserved, scratch
      sup.u(ra.header, 8);
      sup.u(1, 4);
      sup.u(0, 4);
      sup.u(ra.btree, 8);
      sup.u(ra.heap, 8);
      ok = ok && std::fseek(f, (long)sb, SEEK_SET) == 0 && write_all(f, sup.b.data(), sup.b.size());
    } else {
      const uint64_t e0 = sb + (sbver == 1 ? 28 : 24);  // base address field
      Blob eofb, root;
      eofb.u(eof, 8);
      root.u(ra.header, 8);
      root.u(1, 4);
      root.u(0, 4);
      root.u(ra.btree, 8);
      root.u(ra.heap, 8);
      ok = ok && std::fseek(f, (long)(e0 + 16), SEEK_SET) == 0 && write_all(f, eofb.b.data(), 8);
      ok = ok && std::fseek(f, (long)(e0 + 32 + 8), SEEK_SET) == 0 &&
           write_all(f, root.b.data(), root.b.size());
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MEXCT_OK : set_err(MEXCT_ERR_IO, "mat: writing %s failed", path);
  } catch (const Bad& b) {
    return fail(path, b);
  } catch (const std::bad_alloc&) {
    return set_err(MEXCT_ERR_OOM, "mat: %s: out of host memory", path);
  }
}

}  // namespace mexct
