// Host-side npz input: the data format the reference's example loads its
// input from (examples/mnist_pca_tsne.rs:39-44 through npyz 0.9:
// NpzArchive::open, by_name, into_vec).
//
// An .npz file is a ZIP archive of .npy files. This reader follows the
// published formats, written here from their specifications:
//  * ZIP (PKWARE APPNOTE): the end-of-central-directory record (and its ZIP64
//    form), central-directory entries (with ZIP64 extra fields), local headers;
//    entries stored (method 0) or deflated (method 8), checked against their
//    CRC-32;
//  * DEFLATE (RFC 1951): stored, fixed-Huffman and dynamic-Huffman blocks,
//    canonical Huffman codes decoded one bit at a time;
//  * NPY (numpy format versions 1.0 to 3.0): magic, header length, the header
//    dictionary's 'descr', 'fortran_order' and 'shape'.
// Arrays are returned in C order, converted to the dtype's float.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bhtsne_gpu.h"

namespace bhg {
void set_host_error(const std::string& msg);
}

namespace {

struct NpzError {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg) { throw NpzError{code, msg}; }

uint32_t rd16(const std::string& b, size_t p) {
  if (p + 2 > b.size()) fail(BHTSNE_EINVAL, "error: truncated npz archive.");
  return (uint32_t)(uint8_t)b[p] | ((uint32_t)(uint8_t)b[p + 1] << 8);
}
uint32_t rd32(const std::string& b, size_t p) { return rd16(b, p) | (rd16(b, p + 2) << 16); }
uint64_t rd64(const std::string& b, size_t p) { return (uint64_t)rd32(b, p) | ((uint64_t)rd32(b, p + 4) << 32); }

// ---- CRC-32 (polynomial 0xEDB88320, reflected) ------------------------------
uint32_t crc32_of(const uint8_t* p, size_t n) {
  static uint32_t table[256];
  static bool ready = false;
  if (!ready) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    ready = true;
  }
  uint32_t c = 0xFFFFFFFFu;
  for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}

// ---- DEFLATE (RFC 1951) -------------------------------------------------------
struct BitIn {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t acc = 0;
  int nacc = 0;
  uint32_t bits(int k) {  // k <= 16, least significant bit first
    while (nacc < k) {
      if (pos >= n) fail(BHTSNE_EINVAL, "error: truncated deflate stream.");
      acc |= (uint32_t)p[pos++] << nacc;
      nacc += 8;
    }
    const uint32_t v = acc & ((1u << k) - 1u);
    acc >>= k;
    nacc -= k;
    return v;
  }
  void align() {
    acc = 0;
    nacc = 0;
  }
};

// Canonical code of up to 15 bits: per length, the number of codes and the
// symbols in code order (RFC 1951 3.2.2 assigns consecutive codes to the
// symbols of a length in symbol order, shorter lengths first).
struct Huffman {
  uint16_t count[16] = {0};
  std::vector<uint16_t> sym;
  void build(const uint8_t* len, int n) {
    std::memset(count, 0, sizeof count);
    for (int s = 0; s < n; ++s) ++count[len[s]];
    count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
      left = 2 * left - count[l];
      if (left < 0) fail(BHTSNE_EINVAL, "error: over-subscribed Huffman code in a deflate stream.");
    }
    uint16_t off[16];
    off[1] = 0;
    for (int l = 1; l < 15; ++l) off[l + 1] = (uint16_t)(off[l] + count[l]);
    sym.assign(n, 0);
    for (int s = 0; s < n; ++s)
      if (len[s]) sym[off[len[s]]++] = (uint16_t)s;
  }
  int decode(BitIn& in) const {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
      code |= (int)in.bits(1);  // codes are stored most significant bit first
      const int c = count[l];
      if (code < first + c) return sym[index + (code - first)];
      index += c;
      first = (first + c) << 1;
      code <<= 1;
    }
    fail(BHTSNE_EINVAL, "error: invalid Huffman code in a deflate stream.");
  }
};

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_codes(BitIn& in, const Huffman& lit, const Huffman& dist, std::string& out, size_t limit) {
  for (;;) {
    const int s = lit.decode(in);
    if (s < 256) {
      out.push_back((char)s);
    } else if (s == 256) {
      return;
    } else {
      const int li = s - 257;
      if (li >= 29) fail(BHTSNE_EINVAL, "error: invalid length code in a deflate stream.");
      const size_t len = kLenBase[li] + in.bits(kLenExtra[li]);
      const int di = dist.decode(in);
      if (di >= 30) fail(BHTSNE_EINVAL, "error: invalid distance code in a deflate stream.");
      const size_t d = kDistBase[di] + in.bits(kDistExtra[di]);
      if (d > out.size()) fail(BHTSNE_EINVAL, "error: distance too far back in a deflate stream.");
      const size_t from = out.size() - d;
      for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);  // overlapping copies repeat
    }
    if (out.size() > limit) fail(BHTSNE_EINVAL, "error: a deflate stream inflates past its recorded size.");
  }
}

std::string inflate(const uint8_t* p, size_t n, size_t expect) {
  BitIn in{p, n};
  std::string out;
  out.reserve(expect);
  bool last = false;
  while (!last) {
    last = in.bits(1) != 0;
    const uint32_t type = in.bits(2);
    if (type == 0) {
      in.align();
      if (in.pos + 4 > n) fail(BHTSNE_EINVAL, "error: truncated stored block.");
      const uint32_t len = (uint32_t)p[in.pos] | ((uint32_t)p[in.pos + 1] << 8);
      const uint32_t nlen = (uint32_t)p[in.pos + 2] | ((uint32_t)p[in.pos + 3] << 8);
      in.pos += 4;
      if ((len ^ 0xFFFFu) != nlen) fail(BHTSNE_EINVAL, "error: corrupt stored block.");
      if (in.pos + len > n) fail(BHTSNE_EINVAL, "error: truncated stored block.");
      out.append(reinterpret_cast<const char*>(p + in.pos), len);
      in.pos += len;
    } else if (type == 1) {
      uint8_t l[288], d[30];
      for (int s = 0; s < 144; ++s) l[s] = 8;
      for (int s = 144; s < 256; ++s) l[s] = 9;
      for (int s = 256; s < 280; ++s) l[s] = 7;
      for (int s = 280; s < 288; ++s) l[s] = 8;
      for (int s = 0; s < 30; ++s) d[s] = 5;
      Huffman lit, dist;
      lit.build(l, 288);
      dist.build(d, 30);
      inflate_codes(in, lit, dist, out, expect);
    } else if (type == 2) {
      const int nlit = (int)in.bits(5) + 257, ndist = (int)in.bits(5) + 1, ncl = (int)in.bits(4) + 4;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int i = 0; i < ncl; ++i) cl[order[i]] = (uint8_t)in.bits(3);
      Huffman clh;
      clh.build(cl, 19);
      uint8_t lens[320] = {0};
      int i = 0;
      while (i < nlit + ndist) {
        const int s = clh.decode(in);
        if (s < 16) {
          lens[i++] = (uint8_t)s;
        } else {
          int rep = 0;
          uint8_t v = 0;
          if (s == 16) {
            if (i == 0) fail(BHTSNE_EINVAL, "error: repeat without a previous length in a deflate stream.");
            v = lens[i - 1];
            rep = 3 + (int)in.bits(2);
          } else if (s == 17) {
            rep = 3 + (int)in.bits(3);
          } else {
            rep = 11 + (int)in.bits(7);
          }
          if (i + rep > nlit + ndist) fail(BHTSNE_EINVAL, "error: too many code lengths in a deflate stream.");
          while (rep--) lens[i++] = v;
        }
      }
      if (lens[256] == 0) fail(BHTSNE_EINVAL, "error: a deflate block without an end-of-block code.");
      Huffman lit, dist;
      lit.build(lens, nlit);
      dist.build(lens + nlit, ndist);
      inflate_codes(in, lit, dist, out, expect);
    } else {
      fail(BHTSNE_EINVAL, "error: invalid deflate block type.");
    }
  }
  return out;
}

// ---- ZIP ------------------------------------------------------------------------
struct Entry {
  std::string name;
  uint32_t method = 0, crc = 0;
  uint64_t csize = 0, usize = 0, local = 0;
};

std::vector<Entry> zip_entries(const std::string& b) {
  if (b.size() < 22) fail(BHTSNE_EINVAL, "error: not an npz archive (too short for a ZIP directory).");
  size_t eocd = std::string::npos;
  const size_t lo = b.size() >= 22 + 65535 ? b.size() - 22 - 65535 : 0;
  for (size_t p = b.size() - 22 + 1; p-- > lo;)
    if (rd32(b, p) == 0x06054b50u) {
      eocd = p;
      break;
    }
  if (eocd == std::string::npos) fail(BHTSNE_EINVAL, "error: not an npz archive (no ZIP end of central directory).");
  uint64_t entries = rd16(b, eocd + 10), cd_off = rd32(b, eocd + 16);
  if (entries == 0xFFFFu || cd_off == 0xFFFFFFFFu) {
    if (eocd < 20 || rd32(b, eocd - 20) != 0x07064b50u) fail(BHTSNE_EINVAL, "error: ZIP64 locator missing.");
    const uint64_t z64 = rd64(b, eocd - 20 + 8);
    if (z64 + 56 > b.size() || rd32(b, (size_t)z64) != 0x06064b50u) fail(BHTSNE_EINVAL, "error: bad ZIP64 record.");
    entries = rd64(b, (size_t)z64 + 32);
    cd_off = rd64(b, (size_t)z64 + 48);
  }
  std::vector<Entry> out;
  size_t p = (size_t)cd_off;
  for (uint64_t e = 0; e < entries; ++e) {
    if (rd32(b, p) != 0x02014b50u) fail(BHTSNE_EINVAL, "error: corrupt ZIP central directory.");
    Entry en;
    en.method = rd16(b, p + 10);
    en.crc = rd32(b, p + 16);
    en.csize = rd32(b, p + 20);
    en.usize = rd32(b, p + 24);
    const uint32_t nl = rd16(b, p + 28), xl = rd16(b, p + 30), cl = rd16(b, p + 32);
    en.local = rd32(b, p + 42);
    if (p + 46 + nl + xl > b.size()) fail(BHTSNE_EINVAL, "error: truncated ZIP central directory.");
    en.name = b.substr(p + 46, nl);
    // ZIP64 extra field: the 64-bit forms of the fields saturated above, in order
    size_t x = p + 46 + nl;
    const size_t xe = x + xl;
    while (x + 4 <= xe) {
      const uint32_t id = rd16(b, x), sz = rd16(b, x + 2);
      if (id == 0x0001u) {
        size_t q = x + 4;
        if (en.usize == 0xFFFFFFFFu) { en.usize = rd64(b, q); q += 8; }
        if (en.csize == 0xFFFFFFFFu) { en.csize = rd64(b, q); q += 8; }
        if (en.local == 0xFFFFFFFFu) { en.local = rd64(b, q); q += 8; }
      }
      x += 4 + sz;
    }
    out.push_back(en);
    p += 46 + nl + xl + cl;
  }
  return out;
}

std::string zip_read(const std::string& b, const Entry& e) {
  const size_t p = (size_t)e.local;
  if (rd32(b, p) != 0x04034b50u) fail(BHTSNE_EINVAL, "error: corrupt ZIP local header.");
  const size_t data = p + 30 + rd16(b, p + 26) + rd16(b, p + 28);
  if (data + e.csize > b.size()) fail(BHTSNE_EINVAL, "error: truncated ZIP entry.");
  const uint8_t* src = reinterpret_cast<const uint8_t*>(b.data()) + data;
  std::string out;
  if (e.method == 0) {
    out.assign(reinterpret_cast<const char*>(src), (size_t)e.csize);
  } else if (e.method == 8) {
    out = inflate(src, (size_t)e.csize, (size_t)e.usize);
  } else {
    fail(BHTSNE_EINVAL, "error: unsupported ZIP compression method " + std::to_string(e.method) + ".");
  }
  if (out.size() != e.usize) fail(BHTSNE_EINVAL, "error: a ZIP entry's size does not match its directory record.");
  if (crc32_of(reinterpret_cast<const uint8_t*>(out.data()), out.size()) != e.crc)
    fail(BHTSNE_EINVAL, "error: CRC-32 mismatch in npz entry " + e.name + ".");
  return out;
}

// ---- NPY ------------------------------------------------------------------------
struct Npy {
  char kind = 0;  // 'f', 'i', 'u', 'b'
  int size = 0;   // bytes per element
  bool fortran = false;
  std::vector<int64_t> shape;
  size_t data = 0;  // offset of the first element
};

Npy npy_header(const std::string& b) {
  if (b.size() < 10 || std::memcmp(b.data(), "\x93NUMPY", 6) != 0) fail(BHTSNE_EINVAL, "error: not an .npy array.");
  const int major = (uint8_t)b[6];
  size_t hl, h0;
  if (major == 1) {
    hl = rd16(b, 8);
    h0 = 10;
  } else if (major == 2 || major == 3) {
    hl = rd32(b, 8);
    h0 = 12;
  } else {
    fail(BHTSNE_EINVAL, "error: unsupported .npy format version " + std::to_string(major) + ".");
  }
  if (h0 + hl > b.size()) fail(BHTSNE_EINVAL, "error: truncated .npy header.");
  const std::string h = b.substr(h0, hl);
  Npy a;
  a.data = h0 + hl;
  auto value_of = [&](const char* key) -> size_t {
    size_t k = h.find(std::string("'") + key + "'");
    if (k == std::string::npos) k = h.find(std::string("\"") + key + "\"");
    if (k == std::string::npos) fail(BHTSNE_EINVAL, std::string("error: .npy header without '") + key + "'.");
    k = h.find(':', k);
    if (k == std::string::npos) fail(BHTSNE_EINVAL, "error: malformed .npy header.");
    ++k;
    while (k < h.size() && h[k] == ' ') ++k;
    return k;
  };
  size_t d = value_of("descr");
  const char q = h[d];
  if (q != '\'' && q != '"') fail(BHTSNE_EINVAL, "error: unsupported .npy dtype (a structured type).");
  const size_t de = h.find(q, d + 1);
  const std::string descr = h.substr(d + 1, de - d - 1);
  if (descr.size() < 3 || (descr[0] != '<' && descr[0] != '|' && descr[0] != '='))
    fail(BHTSNE_EINVAL, "error: unsupported .npy dtype '" + descr + "' (little-endian numbers only).");
  a.kind = descr[1];
  a.size = std::atoi(descr.c_str() + 2);
  const bool ok = (a.kind == 'f' && (a.size == 4 || a.size == 8)) ||
                  ((a.kind == 'i' || a.kind == 'u') && (a.size == 1 || a.size == 2 || a.size == 4 || a.size == 8)) ||
                  (a.kind == 'b' && a.size == 1);
  if (!ok) fail(BHTSNE_EINVAL, "error: unsupported .npy dtype '" + descr + "'.");
  const size_t f = value_of("fortran_order");
  a.fortran = h.compare(f, 4, "True") == 0;
  size_t s = value_of("shape");
  if (h[s] != '(') fail(BHTSNE_EINVAL, "error: malformed .npy shape.");
  ++s;
  for (;;) {
    while (s < h.size() && (h[s] == ' ' || h[s] == ',')) ++s;
    if (s >= h.size()) fail(BHTSNE_EINVAL, "error: malformed .npy shape.");
    if (h[s] == ')') break;
    int64_t v = 0;
    bool digit = false;
    while (s < h.size() && h[s] >= '0' && h[s] <= '9') {
      v = v * 10 + (h[s++] - '0');
      digit = true;
    }
    while (s < h.size() && h[s] == 'L') ++s;
    if (!digit) fail(BHTSNE_EINVAL, "error: malformed .npy shape.");
    a.shape.push_back(v);
  }
  return a;
}

template <class T>
T element(const uint8_t* p, const Npy& a) {
  uint64_t u = 0;
  for (int k = 0; k < a.size; ++k) u |= (uint64_t)p[k] << (8 * k);
  switch (a.kind) {
    case 'f':
      if (a.size == 4) {
        uint32_t w = (uint32_t)u;
        float f;
        std::memcpy(&f, &w, 4);
        return (T)f;
      } else {
        double g;
        std::memcpy(&g, &u, 8);
        return (T)g;
      }
    case 'i': {
      const int sh = 64 - 8 * a.size;
      const int64_t v = (int64_t)(u << sh) >> sh;  // sign extension
      return (T)v;
    }
    case 'u':
      return (T)u;
    default:
      return (T)(u != 0);
  }
}

template <class T>
void npz_load_impl(const char* path, const char* name, T* out, int64_t* count, int32_t* ndim, int64_t* shape) {
  FILE* fp = std::fopen(path, "rb");
  if (!fp) fail(BHTSNE_EIO, std::string("error: cannot open ") + path + ".");
  std::string buf;
  char chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof chunk, fp)) > 0) buf.append(chunk, got);
  const bool bad = std::ferror(fp) != 0;
  std::fclose(fp);
  if (bad) fail(BHTSNE_EIO, std::string("error: cannot read ") + path + ".");
  const std::vector<Entry> es = zip_entries(buf);
  const std::string want = std::string(name) + ".npy";
  const Entry* hit = nullptr;
  for (const Entry& e : es)
    if (e.name == want || e.name == name) hit = &e;
  if (!hit) fail(BHTSNE_EINVAL, std::string("error: the npz archive has no array '") + name + "'.");
  const std::string arr = zip_read(buf, *hit);
  const Npy a = npy_header(arr);
  int64_t total = 1;
  for (int64_t v : a.shape) total *= v;
  if ((int64_t)a.data + total * a.size > (int64_t)arr.size()) fail(BHTSNE_EINVAL, "error: truncated .npy data.");
  if (ndim) *ndim = (int32_t)a.shape.size();
  if (shape)
    for (size_t k = 0; k < a.shape.size() && k < 8; ++k) shape[k] = a.shape[k];
  if (!out) {
    *count = total;
    return;
  }
  if (*count < total) fail(BHTSNE_EINVAL, "error: the output buffer is too small.");
  const uint8_t* src = reinterpret_cast<const uint8_t*>(arr.data()) + a.data;
  const int nd = (int)a.shape.size();
  if (!a.fortran || nd < 2) {
    for (int64_t e = 0; e < total; ++e) out[e] = element<T>(src + e * a.size, a);
  } else {
    // column-major storage: element (i_0, .., i_{nd-1}) at sum i_k prod_{j<k} n_j
    std::vector<int64_t> idx(nd, 0), stride(nd, 1);
    for (int k = 1; k < nd; ++k) stride[k] = stride[k - 1] * a.shape[k - 1];
    for (int64_t e = 0; e < total; ++e) {
      int64_t off = 0;
      for (int k = 0; k < nd; ++k) off += idx[k] * stride[k];
      out[e] = element<T>(src + off * a.size, a);
      for (int k = nd - 1; k >= 0; --k) {  // next index in C order
        if (++idx[k] < a.shape[k]) break;
        idx[k] = 0;
      }
    }
  }
  *count = total;
}

}  // namespace

extern "C" int bhtsne_load_npz(const char* path, const char* name, int dtype, void* out, int64_t* count, int32_t* ndim,
                               int64_t* shape) {
  try {
    if (!path || !name || !count) fail(BHTSNE_EINVAL, "error: invalid load_npz arguments.");
    if (dtype == BHTSNE_F32) npz_load_impl<float>(path, name, (float*)out, count, ndim, shape);
    else if (dtype == BHTSNE_F64) npz_load_impl<double>(path, name, (double*)out, count, ndim, shape);
    else fail(BHTSNE_EINVAL, "error: dtype must be BHTSNE_F32 or BHTSNE_F64.");
  } catch (const NpzError& e) {
    bhg::set_host_error(e.msg);
    return e.code;
  } catch (const std::exception& e) {
    bhg::set_host_error(std::string("error: ") + e.what());
    return BHTSNE_EINTERNAL;
  }
  return BHTSNE_OK;
}
