// Scanner data files on the host: VFF volumes and MATLAB Level 5 MAT-files.
//
// No counterpart in the reference, whose data files (.vff, .mat) are read in
// MATLAB and kept out of its repository (.gitignore:14-16).  These readers
// feed the same arrays the entry points take (float32, column-major):
//  - VFF: an "ncaa" text header of key=value; lines ended by a form feed,
//    then the raw slices, big-endian (bits 8: unsigned, 16: signed, 32:
//    IEEE float).  The data are the file's last X*Y*Z*bits/8 bytes.
//  - MAT (Level 5, the format of MATLAB's save up to -v7): a 128-byte header,
//    then one data element per variable, either a miMATRIX or a miCOMPRESSED
//    element (zlib stream) holding one.  Numeric classes of any storage type
//    are converted to float32 (real part).  -v7.3 files are HDF5 and are
//    read by mat73.cpp.  Compressed elements (and HDF5's deflated chunks) are
//    inflated by the DEFLATE decoder below, written from RFC 1951 (block
//    formats, canonical Huffman codes, length / distance tables) and RFC 1950
//    (zlib header, Adler-32 check).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mexct.h"
#include "fileio_internal.h"

namespace mexct {
mexct_status set_err(mexct_status code, const char* fmt, ...);
}
using mexct::set_err;

namespace {

bool read_file(const char* path, std::vector<uint8_t>& buf) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  buf.clear();
  // one read of the whole file where its size is known (a scan is GBs), then
  // whatever follows (a file that grew, or one that cannot seek) in pieces
  if (std::fseek(f, 0, SEEK_END) == 0) {
    const long size = std::ftell(f);
    if (size > 0 && std::fseek(f, 0, SEEK_SET) == 0) {
      buf.resize((size_t)size);
      buf.resize(std::fread(buf.data(), 1, buf.size(), f));
    } else {
      std::rewind(f);
    }
  }
  uint8_t chunk[1 << 16];
  size_t n;
  while ((n = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
  const bool ok = !std::ferror(f);
  std::fclose(f);
  return ok;
}

// ---------------------------------------------------------------------------
// DEFLATE (RFC 1951) and the zlib wrapper (RFC 1950)
// ---------------------------------------------------------------------------
constexpr int kFastBits = 9;  // codes up to this length decode with one table lookup

struct Huffman {
  int count[16];  // codes of each length
  int symbol[320];  // symbols in canonical code order
  // the next kFastBits input bits -> symbol and code length (0: a longer
  // code, decoded bit by bit)
  int16_t fast_sym[1 << kFastBits];
  uint8_t fast_len[1 << kFastBits];
};

class Inflater {
 public:
  Inflater(const uint8_t* p, size_t n) : p_(p), n_(n) {}

  // Decodes blocks until the final one; false on malformed or truncated input.
  bool run(std::vector<uint8_t>& out) {
    // out is grown ahead of the writes (bytes [0, used_) are the output) and
    // trimmed once at the end
    used_ = out.size();
    int last;
    bool ok = true;
    do {
      last = (int)bits(1);
      const int type = (int)bits(2);
      if (bad_) {
        ok = false;
        break;
      }
      if (type == 0) ok = stored(out);
      else if (type == 1) ok = fixed(out);
      else if (type == 2) ok = dynamic(out);
      else ok = false;
      if (!ok || bad_) {
        ok = false;
        break;
      }
    } while (!last);
    out.resize(used_);
    return ok;
  }
  size_t consumed() const { return pos_ - (size_t)(cnt_ / 8); }

 private:
  const uint8_t* p_;
  size_t n_, pos_ = 0, used_ = 0;
  uint64_t buf_ = 0;
  int cnt_ = 0;
  bool bad_ = false;

  // k (0..16) bits, least significant first
  uint32_t bits(int k) {
    while (cnt_ < k) {
      if (pos_ >= n_) {
        bad_ = true;
        return 0;
      }
      buf_ |= (uint64_t)p_[pos_++] << cnt_;
      cnt_ += 8;
    }
    const uint32_t v = (uint32_t)(buf_ & ((1ull << k) - 1));
    buf_ >>= k;
    cnt_ -= k;
    return v;
  }

  // Canonical code from code lengths: < 0 over-subscribed, else the number
  // of unused codes (0: complete).
  static int build(Huffman& h, const uint8_t* len, int n) {
    for (int l = 0; l < 16; ++l) h.count[l] = 0;
    std::memset(h.fast_len, 0, sizeof h.fast_len);
    for (int s = 0; s < n; ++s) h.count[len[s]]++;
    if (h.count[0] == n) return 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
      left <<= 1;
      left -= h.count[l];
      if (left < 0) return -1;
    }
    int offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
    for (int s = 0; s < n; ++s)
      if (len[s]) h.symbol[offs[len[s]]++] = s;
    // Lookup table: symbol s of length l <= kFastBits has the canonical code
    // next[l]++ (most significant bit first); the stream holds it reversed,
    // so every table index whose low l bits are the reversed code maps to s.
    if (left == 0) {
      int next[16];
      int code = 0;
      next[0] = 0;
      for (int l = 1; l < 16; ++l) {
        code = (code + h.count[l - 1] * (l > 1)) << 1;
        next[l] = code;
      }
      for (int s = 0; s < n; ++s) {
        const int l = len[s];
        if (l == 0) continue;
        const int c = next[l]++;
        if (l > kFastBits) continue;
        int r = 0;
        for (int b = 0; b < l; ++b) r |= ((c >> b) & 1) << (l - 1 - b);
        for (int fill = 0; fill < (1 << (kFastBits - l)); ++fill) {
          h.fast_sym[r | (fill << l)] = (int16_t)s;
          h.fast_len[r | (fill << l)] = (uint8_t)l;
        }
      }
    }
    return left;
  }

  // One symbol: the code's bits arrive most significant first; codes of
  // each length are consecutive integers starting at `first`.
  int decode(const Huffman& h) {
    while (cnt_ < kFastBits && pos_ < n_) {
      buf_ |= (uint64_t)p_[pos_++] << cnt_;
      cnt_ += 8;
    }
    const int i = (int)(buf_ & ((1u << kFastBits) - 1));
    const int fl = h.fast_len[i];
    if (fl != 0 && fl <= cnt_) {  // only bits that arrived (missing ones read as 0)
      buf_ >>= fl;
      cnt_ -= fl;
      return h.fast_sym[i];
    }
    return decode_slow(h);
  }
  int decode_slow(const Huffman& h) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
      code |= (int)bits(1);
      if (bad_) return -1;
      const int c = h.count[l];
      if (code - first < c) return h.symbol[index + (code - first)];
      index += c;
      first = (first + c) << 1;
      code <<= 1;
    }
    return -1;
  }

  bool stored(std::vector<uint8_t>& out) {
    buf_ >>= (cnt_ & 7);  // to the byte boundary
    cnt_ -= cnt_ & 7;
    const uint32_t len = bits(16), nlen = bits(16);
    if (bad_ || len != (~nlen & 0xffffu)) return false;
    if (out.size() - used_ < len) out.resize(std::max<size_t>(2 * out.size(), used_ + len));
    uint32_t left = len;
    for (; left > 0 && cnt_ >= 8; --left) {  // bytes already in the bit buffer
      out[used_++] = (uint8_t)buf_;
      buf_ >>= 8;
      cnt_ -= 8;
    }
    if (left > n_ - pos_) return false;
    std::memcpy(out.data() + used_, p_ + pos_, left);
    used_ += left;
    pos_ += left;
    return true;
  }

  // Literal / length / distance symbols of one block until its end code.
  // The bit buffer lives in locals here: the output bytes are stored through
  // a uint8_t pointer, which may alias any member, so members would be
  // reloaded after every byte.  The slow (long-code) path and the extra-bit
  // reads at the end of the input go through the members.
  bool codes(std::vector<uint8_t>& out, const Huffman& lit, const Huffman& dist) {
    static const uint16_t lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                       31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                     2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t dbase[30] = {1,    2,    3,    4,    5,    7,     9,     13,    17,  25,
                                       33,   49,   65,   97,   129,  193,   257,   385,   513, 769,
                                       1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                     6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    const uint8_t* const in = p_;
    const size_t n = n_;
    uint64_t buf = buf_;
    int cnt = cnt_;
    size_t pos = pos_;
    size_t size = used_;
    uint8_t* w = out.data();
    size_t cap = out.size();
    auto refill = [&] {
      while (cnt <= 56 && pos < n) {
        buf |= (uint64_t)in[pos++] << cnt;
        cnt += 8;
      }
    };
    auto save = [&] {
      buf_ = buf;
      cnt_ = cnt;
      pos_ = pos;
    };
    auto load = [&] {
      buf = buf_;
      cnt = cnt_;
      pos = pos_;
    };
    auto sym_of = [&](const Huffman& h) -> int {
      refill();
      const int i = (int)(buf & ((1u << kFastBits) - 1));
      const int fl = h.fast_len[i];
      if (fl != 0 && fl <= cnt) {  // only bits that arrived (missing ones read as 0)
        buf >>= fl;
        cnt -= fl;
        return h.fast_sym[i];
      }
      save();
      const int v = decode_slow(h);
      load();
      return v;
    };
    auto extra = [&](int k) -> uint32_t {  // k <= 13 bits
      refill();
      if (cnt < k) {
        bad_ = true;
        return 0;
      }
      const uint32_t v = (uint32_t)(buf & ((1u << k) - 1));
      buf >>= k;
      cnt -= k;
      return v;
    };
    bool ok = false;
    for (;;) {
      if (cap - size < 258) {  // room for the longest match
        out.resize(std::max<size_t>(2 * cap, size + (1u << 16)));
        w = out.data();
        cap = out.size();
      }
      int sym = sym_of(lit);
      if (sym < 0) break;
      if (sym < 256) {
        w[size++] = (uint8_t)sym;
        continue;
      }
      if (sym == 256) {
        ok = true;
        break;
      }
      sym -= 257;
      if (sym >= 29) break;
      const size_t len = (size_t)lbase[sym] + extra(lext[sym]);
      const int ds = sym_of(dist);
      if (ds < 0 || ds >= 30) break;
      const size_t d = (size_t)dbase[ds] + extra(dext[ds]);
      if (bad_ || d > size) break;
      uint8_t* to = w + size;
      const uint8_t* from = to - d;
      for (size_t i = 0; i < len; ++i) to[i] = from[i];  // may overlap: byte by byte
      size += len;
    }
    save();
    used_ = size;
    return ok && !bad_;
  }

  struct FixedCodes {
    Huffman lit, dist;
    FixedCodes() {
      uint8_t l[288];
      for (int s = 0; s < 144; ++s) l[s] = 8;
      for (int s = 144; s < 256; ++s) l[s] = 9;
      for (int s = 256; s < 280; ++s) l[s] = 7;
      for (int s = 280; s < 288; ++s) l[s] = 8;
      build(lit, l, 288);
      for (int s = 0; s < 30; ++s) l[s] = 5;
      build(dist, l, 30);
    }
  };

  bool fixed(std::vector<uint8_t>& out) {
    static const FixedCodes fc;  // built once (thread-safe static initialisation)
    return codes(out, fc.lit, fc.dist);
  }

  bool dynamic(std::vector<uint8_t>& out) {
    static const int order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    const int nlen = (int)bits(5) + 257, ndist = (int)bits(5) + 1, ncode = (int)bits(4) + 4;
    if (bad_ || nlen > 286 || ndist > 30) return false;
    uint8_t lengths[320] = {0};
    for (int i = 0; i < ncode; ++i) lengths[order[i]] = (uint8_t)bits(3);
    Huffman lencode;
    if (build(lencode, lengths, 19) != 0) return false;  // must be complete
    int i = 0;
    while (i < nlen + ndist) {
      const int sym = decode(lencode);
      if (sym < 0) return false;
      if (sym < 16) {
        lengths[i++] = (uint8_t)sym;
      } else {
        int rep;
        uint8_t val = 0;
        if (sym == 16) {
          if (i == 0) return false;
          val = lengths[i - 1];
          rep = 3 + (int)bits(2);
        } else if (sym == 17) {
          rep = 3 + (int)bits(3);
        } else {
          rep = 11 + (int)bits(7);
        }
        if (i + rep > nlen + ndist) return false;
        while (rep--) lengths[i++] = val;
      }
    }
    if (bad_ || lengths[256] == 0) return false;  // no end-of-block code
    Huffman lit, dist;
    const int el = build(lit, lengths, nlen);
    if (el < 0 || (el > 0 && nlen - lit.count[0] != 1)) return false;
    const int ed = build(dist, lengths + nlen, ndist);
    if (ed < 0 || (ed > 0 && ndist - dist.count[0] != 1)) return false;
    return codes(out, lit, dist);
  }
};

// Adler-32 (RFC 1950 section 8.2) with the modulo taken once per block: with
// a, b < 65521 at a block's start, after k bytes b <= 65520 (k + 1) + 255 k (k + 1) / 2,
// which stays below 2^32 for k <= 5552.
uint32_t adler32(const uint8_t* p, size_t n) {
  uint32_t a = 1, b = 0;
  while (n > 0) {
    const size_t k = n < 5552 ? n : 5552;
    for (size_t i = 0; i < k; ++i) {
      a += p[i];
      b += a;
    }
    a %= 65521u;
    b %= 65521u;
    p += k;
    n -= k;
  }
  return (b << 16) | a;
}

// zlib stream -> bytes (header checked, no preset dictionary, Adler-32 checked).
bool zlib_inflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out) {
  if (n < 6) return false;
  const int cmf = p[0], flg = p[1];
  if ((cmf & 0x0f) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20))
    return false;
  Inflater inf(p + 2, n - 2);
  out.clear();
  if (!inf.run(out)) return false;
  const size_t end = 2 + inf.consumed();
  if (end + 4 > n) return false;
  const uint32_t want = ((uint32_t)p[end] << 24) | ((uint32_t)p[end + 1] << 16) |
                        ((uint32_t)p[end + 2] << 8) | (uint32_t)p[end + 3];
  return adler32(out.data(), out.size()) == want;
}

// ---------------------------------------------------------------------------
// MAT-file Level 5
// ---------------------------------------------------------------------------
enum MiType {
  miINT8 = 1, miUINT8 = 2, miINT16 = 3, miUINT16 = 4, miINT32 = 5, miUINT32 = 6, miSINGLE = 7,
  miDOUBLE = 9, miINT64 = 12, miUINT64 = 13, miMATRIX = 14, miCOMPRESSED = 15, miUTF8 = 16,
  miUTF16 = 17, miUTF32 = 18
};

int mi_size(int t) {
  switch (t) {
    case miINT8: case miUINT8: case miUTF8: return 1;
    case miINT16: case miUINT16: case miUTF16: return 2;
    case miINT32: case miUINT32: case miSINGLE: case miUTF32: return 4;
    case miDOUBLE: case miINT64: case miUINT64: return 8;
    default: return 0;
  }
}

struct Reader {
  const uint8_t* p;
  size_t n;
  bool swap;
  uint32_t u32(size_t o) const {
    uint32_t v;
    std::memcpy(&v, p + o, 4);
    return swap ? __builtin_bswap32(v) : v;
  }
};

struct Element {
  int type = 0;
  const uint8_t* data = nullptr;
  size_t nbytes = 0;
  size_t next = 0;  // offset of the following element
};

bool element_at(const Reader& r, size_t off, Element& e) {
  if (off + 8 > r.n) return false;
  const uint32_t t0 = r.u32(off);
  if (t0 >> 16) {  // small data element: type and size share the first word
    e.type = (int)(t0 & 0xffff);
    e.nbytes = t0 >> 16;
    if (e.nbytes > 4) return false;
    e.data = r.p + off + 4;
    e.next = off + 8;
    return true;
  }
  e.type = (int)t0;
  e.nbytes = r.u32(off + 4);
  if (off + 8 + e.nbytes > r.n) return false;
  e.data = r.p + off + 8;
  // elements are padded to 8 bytes; a compressed element is not
  e.next = off + 8 + (e.type == miCOMPRESSED ? e.nbytes : (e.nbytes + 7) / 8 * 8);
  if (e.next > r.n) e.next = r.n;
  return true;
}

double mi_value(const uint8_t* p, int type, bool swap) {
  uint8_t b[8];
  const int s = mi_size(type);
  for (int i = 0; i < s; ++i) b[i] = swap ? p[s - 1 - i] : p[i];
  switch (type) {
    case miINT8: { int8_t v; std::memcpy(&v, b, 1); return v; }
    case miUINT8: return b[0];
    case miINT16: { int16_t v; std::memcpy(&v, b, 2); return v; }
    case miUINT16: { uint16_t v; std::memcpy(&v, b, 2); return v; }
    case miINT32: { int32_t v; std::memcpy(&v, b, 4); return v; }
    case miUINT32: { uint32_t v; std::memcpy(&v, b, 4); return v; }
    case miSINGLE: { float v; std::memcpy(&v, b, 4); return v; }
    case miDOUBLE: { double v; std::memcpy(&v, b, 8); return v; }
    case miINT64: { int64_t v; std::memcpy(&v, b, 8); return (double)v; }
    case miUINT64: { uint64_t v; std::memcpy(&v, b, 8); return (double)v; }
    default: return 0.0;
  }
}

struct MatVar {
  std::string name;
  int mclass = 0;
  bool numeric = false;
  std::vector<long long> dims;
  Element real;
  bool swap = false;
};

// A miMATRIX element's array flags, dims, name and real part.
bool parse_matrix(const Reader& r, const Element& m, MatVar& v) {
  Reader s{m.data, m.nbytes, r.swap};
  Element f, d, nm;
  if (!element_at(s, 0, f) || f.type != miUINT32 || f.nbytes < 8) return false;
  const uint32_t flags = Reader{f.data, 8, r.swap}.u32(0);
  v.mclass = (int)(flags & 0xff);
  v.numeric = v.mclass >= 6 && v.mclass <= 15;  // mxDOUBLE .. mxUINT64
  if (!element_at(s, f.next, d) || d.type != miINT32) return false;
  v.dims.clear();
  for (size_t i = 0; i + 4 <= d.nbytes; i += 4) {
    int32_t x;
    uint32_t u = Reader{d.data, d.nbytes, r.swap}.u32(i);
    std::memcpy(&x, &u, 4);
    v.dims.push_back(x);
  }
  if (!element_at(s, d.next, nm) || nm.type != miINT8) return false;
  v.name.assign(reinterpret_cast<const char*>(nm.data), nm.nbytes);
  v.swap = r.swap;
  if (v.numeric) {
    if (!element_at(s, nm.next, v.real) || mi_size(v.real.type) == 0) return false;
  }
  return true;
}

struct MatFile {
  std::vector<uint8_t> raw;
  std::vector<std::vector<uint8_t>> inflated;  // storage of decompressed variables
  std::vector<MatVar> vars;
  bool h5 = false;  // a -v7.3 (HDF5) file: its variables are in h5vars
  std::vector<mexct::Mat73Var> h5vars;
};

mexct_status load_mat(const char* path, MatFile& mf) {
  if (!path) return set_err(MEXCT_ERR_ARG, "mat: NULL path");
  if (!read_file(path, mf.raw)) return set_err(MEXCT_ERR_IO, "mat: cannot read %s", path);
  if (mf.raw.size() < 128) return set_err(MEXCT_ERR_IO, "mat: %s is not a MAT-file", path);
  if (std::memcmp(mf.raw.data(), "MATLAB 7.3", 10) == 0 || mexct::mat73_is_hdf5(mf.raw)) {
    mf.h5 = true;
    return mexct::mat73_list(mf.raw, path, mf.h5vars);
  }
  const char e0 = (char)mf.raw[126], e1 = (char)mf.raw[127];
  bool swap;
  if (e0 == 'I' && e1 == 'M') swap = false;       // written little-endian
  else if (e0 == 'M' && e1 == 'I') swap = true;   // written big-endian
  else return set_err(MEXCT_ERR_IO, "mat: %s has no Level 5 header", path);
  Reader r{mf.raw.data(), mf.raw.size(), swap};
  size_t off = 128;
  mf.inflated.reserve(64);
  while (off + 8 <= r.n) {
    Element e;
    if (!element_at(r, off, e)) return set_err(MEXCT_ERR_IO, "mat: %s is truncated", path);
    if (e.type == miCOMPRESSED) {
      mf.inflated.emplace_back();
      std::vector<uint8_t>& buf = mf.inflated.back();
      if (!zlib_inflate(e.data, e.nbytes, buf))
        return set_err(MEXCT_ERR_IO, "mat: a compressed variable of %s does not inflate", path);
      Reader z{buf.data(), buf.size(), swap};
      Element inner;
      if (!element_at(z, 0, inner))
        return set_err(MEXCT_ERR_IO, "mat: %s: bad compressed element", path);
      if (inner.type == miMATRIX) {
        MatVar v;
        if (!parse_matrix(z, inner, v)) return set_err(MEXCT_ERR_IO, "mat: %s: bad array", path);
        mf.vars.push_back(v);
      }
    } else if (e.type == miMATRIX) {
      MatVar v;
      if (!parse_matrix(r, e, v)) return set_err(MEXCT_ERR_IO, "mat: %s: bad array", path);
      mf.vars.push_back(v);
    }
    off = e.next;
  }
  return MEXCT_OK;
}

mexct_status find_var(const MatFile& mf, const char* path, const char* name, const MatVar** out) {
  for (const MatVar& v : mf.vars) {
    if (name && *name) {
      if (v.name == name) {
        if (!v.numeric)
          return set_err(MEXCT_ERR_UNSUPPORTED, "mat: %s in %s is not a numeric array", name, path);
        *out = &v;
        return MEXCT_OK;
      }
    } else if (v.numeric) {
      *out = &v;
      return MEXCT_OK;
    }
  }
  if (name && *name) return set_err(MEXCT_ERR_ARG, "mat: no variable %s in %s", name, path);
  return set_err(MEXCT_ERR_ARG, "mat: no numeric variable in %s", path);
}

mexct_status find_var73(const MatFile& mf, const char* path, const char* name,
                        const mexct::Mat73Var** out) {
  for (const mexct::Mat73Var& v : mf.h5vars) {
    if (name && *name) {
      if (v.name == name) {
        if (v.unsupported)
          return set_err(MEXCT_ERR_UNSUPPORTED, "mat: %s in %s (-v7.3 / HDF5): %s", name, path,
                         v.unsupported);
        if (!v.numeric)
          return set_err(MEXCT_ERR_UNSUPPORTED, "mat: %s in %s is not a numeric array (%s)", name,
                         path, v.mclass.empty() ? "group" : v.mclass.c_str());
        *out = &v;
        return MEXCT_OK;
      }
    } else if (v.numeric) {
      *out = &v;
      return MEXCT_OK;
    }
  }
  if (name && *name) return set_err(MEXCT_ERR_ARG, "mat: no variable %s in %s", name, path);
  return set_err(MEXCT_ERR_ARG, "mat: no numeric variable in %s", path);
}

void put_u32(std::vector<uint8_t>& b, uint32_t v) {
  for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
void pad8(std::vector<uint8_t>& b) {
  while (b.size() % 8) b.push_back(0);
}

// ---------------------------------------------------------------------------
// VFF
// ---------------------------------------------------------------------------
struct VffInfo {
  int dims[3] = {0, 0, 1};
  float spacing[3] = {1.f, 1.f, 1.f};
  int bits = 0;
  size_t data_off = 0;
};

mexct_status parse_vff(const std::vector<uint8_t>& f, const char* path, VffInfo& vi) {
  if (f.size() < 5 || std::memcmp(f.data(), "ncaa", 4) != 0)
    return set_err(MEXCT_ERR_IO, "vff: %s does not start with ncaa", path);
  size_t end = 0;
  while (end < f.size() && f[end] != 0x0c) ++end;
  if (end == f.size()) return set_err(MEXCT_ERR_IO, "vff: %s: header has no form feed", path);
  const std::string hdr(reinterpret_cast<const char*>(f.data()), end);
  int rank = 3, bands = 1, nsize = 0;
  std::string format = "slice", type = "raster";
  size_t pos = hdr.find('\n');
  while (pos != std::string::npos && pos < hdr.size()) {
    const size_t stop = hdr.find_first_of(";\n", pos + 1);
    std::string line = hdr.substr(pos + 1, (stop == std::string::npos ? hdr.size() : stop) - pos - 1);
    pos = stop == std::string::npos ? stop : hdr.find('\n', stop);
    const size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    std::string key = line.substr(0, eq), val = line.substr(eq + 1);
    while (!key.empty() && (key.back() == ' ' || key.back() == '\r')) key.pop_back();
    while (!key.empty() && (key[0] == ' ' || key[0] == '\r')) key.erase(0, 1);
    if (key == "rank") rank = std::atoi(val.c_str());
    else if (key == "bands") bands = std::atoi(val.c_str());
    else if (key == "bits") vi.bits = std::atoi(val.c_str());
    else if (key == "format") format = val.substr(0, val.find_first_of(" \r"));
    else if (key == "type") type = val.substr(0, val.find_first_of(" \r"));
    else if (key == "size")
      nsize = std::sscanf(val.c_str(), "%d %d %d", &vi.dims[0], &vi.dims[1], &vi.dims[2]);
    else if (key == "spacing")
      std::sscanf(val.c_str(), "%f %f %f", &vi.spacing[0], &vi.spacing[1], &vi.spacing[2]);
  }
  if (type != "raster" || format != "slice" || bands != 1 || (rank != 2 && rank != 3))
    return set_err(MEXCT_ERR_UNSUPPORTED,
                   "vff: %s: only single-band raster slices of rank 2 or 3 are read", path);
  if (nsize < 2 || vi.dims[0] < 1 || vi.dims[1] < 1 || vi.dims[2] < 1)
    return set_err(MEXCT_ERR_IO, "vff: %s: bad size", path);
  if (rank == 2) vi.dims[2] = 1;
  if (vi.bits != 8 && vi.bits != 16 && vi.bits != 32)
    return set_err(MEXCT_ERR_UNSUPPORTED, "vff: %s: bits=%d (8, 16 or 32 are read)", path, vi.bits);
  const size_t bytes = (size_t)vi.dims[0] * vi.dims[1] * vi.dims[2] * (vi.bits / 8);
  if (f.size() < end + 1 + bytes) return set_err(MEXCT_ERR_IO, "vff: %s is truncated", path);
  vi.data_off = f.size() - bytes;
  return MEXCT_OK;
}

}  // namespace

namespace mexct {
bool zlib_inflate_bytes(const uint8_t* p, size_t n, std::vector<uint8_t>& out) {
  return zlib_inflate(p, n, out);
}
}  // namespace mexct

extern "C" {

mexct_status mexct_mat_list(const char* path, char* names, size_t capacity) {
  MatFile mf;
  if (mexct_status s = load_mat(path, mf)) return s;
  std::string all;
  for (const MatVar& v : mf.vars) {
    if (!all.empty()) all += '\n';
    all += v.name;
  }
  for (const mexct::Mat73Var& v : mf.h5vars) {
    if (!all.empty()) all += '\n';
    all += v.name;
  }
  if (!names || capacity < all.size() + 1)
    return set_err(MEXCT_ERR_ARG, "mat: the name list needs %zu bytes", all.size() + 1);
  std::memcpy(names, all.c_str(), all.size() + 1);
  return MEXCT_OK;
}

mexct_status mexct_mat_info(const char* path, const char* name, int* ndims, long long* dims) {
  if (!ndims || !dims) return set_err(MEXCT_ERR_ARG, "mat: NULL output");
  MatFile mf;
  if (mexct_status s = load_mat(path, mf)) return s;
  if (mf.h5) {
    const mexct::Mat73Var* v = nullptr;
    if (mexct_status s = find_var73(mf, path, name, &v)) return s;
    if (v->dims.size() > 8) return set_err(MEXCT_ERR_UNSUPPORTED, "mat: more than 8 dimensions");
    *ndims = (int)v->dims.size();
    for (size_t i = 0; i < v->dims.size(); ++i) dims[i] = v->dims[i];
    return MEXCT_OK;
  }
  const MatVar* v = nullptr;
  if (mexct_status s = find_var(mf, path, name, &v)) return s;
  if (v->dims.size() > 8) return set_err(MEXCT_ERR_UNSUPPORTED, "mat: more than 8 dimensions");
  *ndims = (int)v->dims.size();
  for (size_t i = 0; i < v->dims.size(); ++i) dims[i] = v->dims[i];
  return MEXCT_OK;
}

mexct_status mexct_mat_read(const char* path, const char* name, float* out, long long count) {
  MatFile mf;
  if (mexct_status s = load_mat(path, mf)) return s;
  if (mf.h5) {
    const mexct::Mat73Var* v = nullptr;
    if (mexct_status s = find_var73(mf, path, name, &v)) return s;
    return mexct::mat73_read(mf.raw, path, *v, out, count);
  }
  const MatVar* v = nullptr;
  if (mexct_status s = find_var(mf, path, name, &v)) return s;
  long long n = 1;
  for (long long d : v->dims) n *= d;
  const int es = mi_size(v->real.type);
  if ((long long)v->real.nbytes < n * es)
    return set_err(MEXCT_ERR_IO, "mat: %s: data shorter than its dimensions", path);
  if (count != n) return set_err(MEXCT_ERR_ARG, "mat: %s holds %lld elements, not %lld",
                                 v->name.c_str(), n, count);
  if (n > 0 && !out) return set_err(MEXCT_ERR_ARG, "mat: NULL output");
  const uint8_t* src = v->real.data;
  if (v->real.type == miSINGLE && !v->swap) {  // the common cases in bulk
    std::memcpy(out, src, 4 * (size_t)n);
  } else if (v->real.type == miDOUBLE && !v->swap) {
    for (long long i = 0; i < n; ++i) {
      double d;
      std::memcpy(&d, src + 8 * i, 8);
      out[i] = (float)d;
    }
  } else {
    for (long long i = 0; i < n; ++i) out[i] = (float)mi_value(src + i * es, v->real.type, v->swap);
  }
  return MEXCT_OK;
}

mexct_status mexct_mat_write(const char* path, const char* name, const float* data, int ndims,
                             const long long* dims, int append) {
  return mexct_mat_write_ex(path, name, data, ndims, dims, append, MEXCT_MAT_AUTO);
}

mexct_status mexct_mat_write_ex(const char* path, const char* name, const float* data, int ndims,
                                const long long* dims, int append, int format) {
  if (!path || !name || !*name || !dims || ndims < 2 || ndims > 8)
    return set_err(MEXCT_ERR_ARG, "mat: bad arguments (name, 2..8 dims)");
  if (format != MEXCT_MAT_AUTO && format != MEXCT_MAT_V5 && format != MEXCT_MAT_V73)
    return set_err(MEXCT_ERR_ARG, "mat: unknown format %d", format);
  unsigned long long total = 1;
  for (int i = 0; i < ndims; ++i) {
    if (dims[i] < 0) return set_err(MEXCT_ERR_ARG, "mat: bad dimension");
    if (dims[i] != 0 && total > (1ull << 40) / (unsigned long long)dims[i])
      return set_err(MEXCT_ERR_ARG, "mat: more than 2^40 elements");
    total *= (unsigned long long)dims[i];
  }
  // the file being appended to decides; else -v7.3 where MATLAB needs it (a
  // variable of 2 GB or more)
  bool existing_h5 = false, existing = false;
  if (append) {
    FILE* g = std::fopen(path, "rb");
    if (g) {
      std::vector<uint8_t> head(1032);
      head.resize(std::fread(head.data(), 1, head.size(), g));
      std::fclose(g);
      existing = head.size() >= 128;
      existing_h5 = existing && (mexct::mat73_is_hdf5(head) ||
                                 std::memcmp(head.data(), "MATLAB 7.3", 10) == 0);
    }
  }
  int fmt = format;
  if (fmt == MEXCT_MAT_AUTO)
    fmt = existing ? (existing_h5 ? MEXCT_MAT_V73 : MEXCT_MAT_V5)
                   : (4 * total >= (1ull << 31) ? MEXCT_MAT_V73 : MEXCT_MAT_V5);
  if (existing && (fmt == MEXCT_MAT_V73) != existing_h5)
    return set_err(MEXCT_ERR_ARG, "mat: %s is a %s file; cannot append a %s variable", path,
                   existing_h5 ? "-v7.3" : "Level 5", fmt == MEXCT_MAT_V73 ? "-v7.3" : "Level 5");
  if (fmt == MEXCT_MAT_V73) return mexct::mat73_write(path, name, data, ndims, dims, existing);
  long long n = 1;
  for (int i = 0; i < ndims; ++i) {
    if (dims[i] > 0x7fffffffLL) return set_err(MEXCT_ERR_ARG, "mat: bad dimension");
    n *= dims[i];
  }
  const size_t nl = std::strlen(name);
  if (nl > 63) return set_err(MEXCT_ERR_ARG, "mat: name longer than 63 characters");
  if (n > 0 && !data) return set_err(MEXCT_ERR_ARG, "mat: NULL data");
  if ((unsigned long long)n * 4 > 0xffffff00ull)
    return set_err(MEXCT_ERR_UNSUPPORTED, "mat: a Level 5 element holds at most 4 GiB");
  std::vector<uint8_t> body;
  put_u32(body, miUINT32);  // array flags: single class, real
  put_u32(body, 8);
  put_u32(body, 7);
  put_u32(body, 0);
  put_u32(body, miINT32);
  put_u32(body, (uint32_t)(4 * ndims));
  for (int i = 0; i < ndims; ++i) put_u32(body, (uint32_t)dims[i]);
  pad8(body);
  put_u32(body, miINT8);
  put_u32(body, (uint32_t)nl);
  body.insert(body.end(), name, name + nl);
  pad8(body);
  put_u32(body, miSINGLE);
  put_u32(body, (uint32_t)(4 * n));
  // the data follow body straight from the caller's array (a little-endian file)
  const size_t tail = (8 - (4 * (size_t)n) % 8) % 8;
  std::vector<uint8_t> elem;
  put_u32(elem, miMATRIX);
  put_u32(elem, (uint32_t)(body.size() + 4 * (size_t)n + tail));
  const bool header = !existing;  // a new file (or one too short to hold a header)
  FILE* f = std::fopen(path, header ? "wb" : "ab");
  if (!f) return set_err(MEXCT_ERR_IO, "mat: cannot write %s", path);
  bool ok = true;
  if (header) {
    char h[128];
    std::memset(h, ' ', 116);
    const char* txt = "MATLAB 5.0 MAT-file, written by mexct-gb300";
    std::memcpy(h, txt, std::strlen(txt));
    std::memset(h + 116, 0, 8);  // no subsystem data
    h[124] = 0x00;               // version 0x0100, little-endian
    h[125] = 0x01;
    h[126] = 'I';
    h[127] = 'M';
    ok = std::fwrite(h, 1, 128, f) == 128;
  }
  const uint8_t zeros[8] = {};
  ok = ok && std::fwrite(elem.data(), 1, elem.size(), f) == elem.size();
  ok = ok && std::fwrite(body.data(), 1, body.size(), f) == body.size();
  ok = ok && (n == 0 || std::fwrite(data, 4, (size_t)n, f) == (size_t)n);
  ok = ok && std::fwrite(zeros, 1, tail, f) == tail;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? MEXCT_OK : set_err(MEXCT_ERR_IO, "mat: writing %s failed", path);
}

mexct_status mexct_vff_info(const char* path, int* dims, float* spacing, int* bits) {
  if (!path || !dims) return set_err(MEXCT_ERR_ARG, "vff: NULL argument");
  std::vector<uint8_t> f;
  if (!read_file(path, f)) return set_err(MEXCT_ERR_IO, "vff: cannot read %s", path);
  VffInfo vi;
  if (mexct_status s = parse_vff(f, path, vi)) return s;
  for (int i = 0; i < 3; ++i) {
    dims[i] = vi.dims[i];
    if (spacing) spacing[i] = vi.spacing[i];
  }
  if (bits) *bits = vi.bits;
  return MEXCT_OK;
}

mexct_status mexct_vff_read(const char* path, float* out, long long count) {
  if (!path) return set_err(MEXCT_ERR_ARG, "vff: NULL path");
  std::vector<uint8_t> f;
  if (!read_file(path, f)) return set_err(MEXCT_ERR_IO, "vff: cannot read %s", path);
  VffInfo vi;
  if (mexct_status s = parse_vff(f, path, vi)) return s;
  const long long n = (long long)vi.dims[0] * vi.dims[1] * vi.dims[2];
  if (count != n) return set_err(MEXCT_ERR_ARG, "vff: %s holds %lld voxels, not %lld", path, n, count);
  if (!out) return set_err(MEXCT_ERR_ARG, "vff: NULL output");
  const uint8_t* p = f.data() + vi.data_off;
  for (long long i = 0; i < n; ++i) {
    if (vi.bits == 8) {
      out[i] = (float)p[i];
    } else if (vi.bits == 16) {
      const uint16_t u = (uint16_t)((p[2 * i] << 8) | p[2 * i + 1]);
      int16_t v;
      std::memcpy(&v, &u, 2);
      out[i] = (float)v;
    } else {
      const uint32_t u = ((uint32_t)p[4 * i] << 24) | ((uint32_t)p[4 * i + 1] << 16) |
                         ((uint32_t)p[4 * i + 2] << 8) | (uint32_t)p[4 * i + 3];
      float v;
      std::memcpy(&v, &u, 4);
      out[i] = v;
    }
  }
  return MEXCT_OK;
}

mexct_status mexct_vff_write(const char* path, const float* data, const int* dims,
                             const float* spacing, int bits) {
  if (!path || !data || !dims) return set_err(MEXCT_ERR_ARG, "vff: NULL argument");
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return set_err(MEXCT_ERR_ARG, "vff: bad size");
  if (bits != 16 && bits != 32) return set_err(MEXCT_ERR_ARG, "vff: bits must be 16 or 32");
  const float sp[3] = {spacing ? spacing[0] : 1.f, spacing ? spacing[1] : 1.f,
                       spacing ? spacing[2] : 1.f};
  const long long n = (long long)dims[0] * dims[1] * dims[2];
  char hdr[512];
  const int len = std::snprintf(hdr, sizeof hdr,
                                "ncaa\nrank=3;\ntype=raster;\nformat=slice;\nbits=%d;\nbands=1;\n"
                                "size=%d %d %d;\nspacing=%g %g %g;\norigin=0 0 0;\n"
                                "rawsize=%lld;\n\f\n",
                                bits, dims[0], dims[1], dims[2], sp[0], sp[1], sp[2],
                                n * (bits / 8));
  std::vector<uint8_t> buf(hdr, hdr + len);
  buf.reserve(buf.size() + (size_t)n * (bits / 8));
  for (long long i = 0; i < n; ++i) {
    if (bits == 16) {
      const float r = std::nearbyint(std::fmin(std::fmax(data[i], -32768.f), 32767.f));
      const int16_t v = (int16_t)(std::isnan(data[i]) ? 0.f : r);
      uint16_t u;
      std::memcpy(&u, &v, 2);
      buf.push_back((uint8_t)(u >> 8));
      buf.push_back((uint8_t)u);
    } else {
      uint32_t u;
      std::memcpy(&u, &data[i], 4);
      for (int k = 3; k >= 0; --k) buf.push_back((uint8_t)(u >> (8 * k)));
    }
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_err(MEXCT_ERR_IO, "vff: cannot write %s", path);
  bool ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? MEXCT_OK : set_err(MEXCT_ERR_IO, "vff: writing %s failed", path);
}

}  // extern "C"
