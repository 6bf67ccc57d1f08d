// Host-side CSV input and output around the fitting path: load_csv and
// tSNE::write_csv of the reference (src/csv.rs:31-118).
//
//  * load_csv reads a comma-separated file with the reader defaults of the csv
//    crate the reference uses: '"' quoting with doubled quotes inside quoted
//    fields, "\n" or "\r\n" record ends, empty lines skipped, every record with
//    the field count of the first (a header record included). Fields not
//    listed in `skip` are parsed as T in file order. The reference converts
//    each field with a caller's closure; the C ABI parses numbers as Rust's
//    str::parse does (an optional sign, decimal or exponent form, inf,
//    infinity and nan in any case; no surrounding whitespace).
//  * write_csv writes the embedding one point per record, with the header
//    "x,y" for D = 2 and "x,y,z" for D = 3, each value as Rust's Display
//    prints a float: the shortest decimal that reads back to the same value,
//    without an exponent ("NaN", "inf" and "-inf" for the non-finite values).
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <system_error>
#include <vector>

#include "../../include/bhtsne_gpu.h"

namespace {

thread_local std::string g_io_error;

int io_fail(int code, const std::string& msg) {
  g_io_error = msg;
  return code;
}

// One CSV record at a time from a whole-file buffer.
struct CsvReader {
  const std::string& buf;
  size_t pos = 0;
  explicit CsvReader(const std::string& b) : buf(b) {}

  // Reads the next non-empty record into fields; false at the end of input.
  bool next(std::vector<std::string>& fields, std::string* err) {
    for (;;) {
      if (pos >= buf.size()) return false;
      // an empty line (bare record terminator) is skipped
      if (buf[pos] == '\n') {
        ++pos;
        continue;
      }
      if (buf[pos] == '\r' && pos + 1 < buf.size() && buf[pos + 1] == '\n') {
        pos += 2;
        continue;
      }
      break;
    }
    fields.clear();
    std::string cur;
    for (;;) {
      if (pos < buf.size() && buf[pos] == '"') {
        // quoted field: up to the closing quote, "" is a literal quote
        ++pos;
        for (;;) {
          if (pos >= buf.size()) {
            *err = "unterminated quoted field";
            return false;
          }
          const char c = buf[pos++];
          if (c == '"') {
            if (pos < buf.size() && buf[pos] == '"') {
              cur.push_back('"');
              ++pos;
            } else {
              break;
            }
          } else {
            cur.push_back(c);
          }
        }
        // anything up to the delimiter after a closing quote belongs to the field
        while (pos < buf.size() && buf[pos] != ',' && buf[pos] != '\n' && buf[pos] != '\r') cur.push_back(buf[pos++]);
      } else {
        while (pos < buf.size() && buf[pos] != ',' && buf[pos] != '\n' && buf[pos] != '\r') cur.push_back(buf[pos++]);
      }
      fields.push_back(cur);
      cur.clear();
      if (pos >= buf.size()) return true;
      if (buf[pos] == ',') {
        ++pos;
        continue;
      }
      if (buf[pos] == '\r') ++pos;
      if (pos < buf.size() && buf[pos] == '\n') ++pos;
      return true;
    }
  }
};

bool ieq(const char* a, size_t n, const char* b) {
  if (std::strlen(b) != n) return false;
  for (size_t i = 0; i < n; ++i) {
    char c = a[i];
    if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
    if (c != b[i]) return false;
  }
  return true;
}

// Rust str::parse::<f32 / f64>: [+-] then a decimal (digits, optional point,
// optional exponent) or inf / infinity / nan, case-insensitively.
template <class T>
bool parse_number(const std::string& s, T* out) {
  const char* p = s.data();
  size_t n = s.size();
  bool neg = false;
  if (n > 0 && (p[0] == '+' || p[0] == '-')) {
    neg = p[0] == '-';
    ++p;
    --n;
  }
  if (n == 0) return false;
  if (ieq(p, n, "inf") || ieq(p, n, "infinity")) {
    *out = neg ? -INFINITY : INFINITY;
    return true;
  }
  if (ieq(p, n, "nan")) {
    *out = (T)NAN;
    return true;
  }
  // digits, '.', digits, optional exponent: from_chars in general form, after
  // checking that nothing else (such as whitespace, a second sign or a hex
  // prefix) is present
  if (!((p[0] >= '0' && p[0] <= '9') || p[0] == '.')) return false;
  for (size_t i = 0; i < n; ++i) {
    const char c = p[i];
    if (!((c >= '0' && c <= '9') || c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-')) return false;
  }
  T v{};
  const auto r = std::from_chars(p, p + n, v, std::chars_format::general);
  if (r.ec == std::errc::result_out_of_range) {
    // Rust rounds overflow to infinity and underflow to zero
    errno = 0;
    const double d = std::strtod(std::string(p, n).c_str(), nullptr);
    v = (T)d;
  } else if (r.ec != std::errc() || r.ptr != p + n) {
    return false;
  }
  *out = neg ? -v : v;
  return true;
}

// Rust's Display of a float: shortest round-trip digits, no exponent.
template <class T>
void format_number(T v, std::string& out) {
  if (std::isnan(v)) {
    out += "NaN";
    return;
  }
  if (std::isinf(v)) {
    out += v < 0 ? "-inf" : "inf";
    return;
  }
  // shortest round-trip digits from the scientific form d.ddd e+-XX, then
  // written out positionally (zeros padded), as Rust formats them
  char buf[64];
  const auto r = std::to_chars(buf, buf + sizeof buf - 1, v, std::chars_format::scientific);
  *r.ptr = '\0';
  const char* p = buf;
  if (*p == '-') {
    out.push_back('-');
    ++p;
  }
  std::string digits;
  while (p < r.ptr && *p != 'e') {
    if (*p != '.') digits.push_back(*p);
    ++p;
  }
  const int exp10 = std::atoi(p + 1);  // value = d.ddd x 10^exp10
  if (exp10 >= 0) {
    const size_t int_len = (size_t)exp10 + 1;
    if (digits.size() <= int_len) {
      out += digits;
      out.append(int_len - digits.size(), '0');
    } else {
      out.append(digits, 0, int_len);
      out.push_back('.');
      out.append(digits, int_len, std::string::npos);
    }
  } else {
    out += "0.";
    out.append((size_t)(-exp10 - 1), '0');
    out += digits;
  }
}

template <class T>
int load_csv_impl(const char* path, int32_t has_headers, const int64_t* skip, int64_t n_skip, T* out,
                  int64_t* count, int64_t* records) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return io_fail(BHTSNE_EIO, std::string("error: cannot open ") + path + ": " + std::strerror(errno));
  std::string buf;
  char chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.append(chunk, got);
  const bool bad = std::ferror(f) != 0;
  std::fclose(f);
  if (bad) return io_fail(BHTSNE_EIO, std::string("error: cannot read ") + path);
  CsvReader rd(buf);
  std::vector<std::string> fields;
  std::string err;
  int64_t nrec = 0, nval = 0, line = 0;
  size_t width = 0;
  bool first = true;
  while (rd.next(fields, &err)) {
    ++line;
    if (first) {
      width = fields.size();
      first = false;
    } else if (fields.size() != width) {
      return io_fail(BHTSNE_EINVAL, "error: CSV error: record " + std::to_string(line) + ": found record with " +
                                        std::to_string(fields.size()) + " fields, but the previous record has " +
                                        std::to_string(width) + " fields");
    }
    if (line == 1 && has_headers) continue;
    for (size_t c = 0; c < fields.size(); ++c) {
      bool skipped = false;
      for (int64_t k = 0; k < n_skip; ++k) skipped = skipped || skip[k] == (int64_t)c;
      if (skipped) continue;
      if (out) {
        T v;
        if (!parse_number<T>(fields[c], &v))
          return io_fail(BHTSNE_EINVAL, "error: record " + std::to_string(line) + ", field " + std::to_string(c) +
                                            ": invalid float literal \"" + fields[c] + "\"");
        if (nval >= *count) return io_fail(BHTSNE_EINVAL, "error: the output buffer is too small.");
        out[nval] = v;
      }
      ++nval;
    }
    ++nrec;
  }
  if (!err.empty()) return io_fail(BHTSNE_EINVAL, "error: CSV error: " + err);
  *count = nval;
  if (records) *records = nrec;
  return BHTSNE_OK;
}

template <class T>
int write_csv_impl(const T* y, int64_t n, int32_t D, const char* path) {
  std::string s;
  if (D == 2) s += "x,y\n";
  else if (D == 3) s += "x,y,z\n";
  for (int64_t i = 0; i < n; ++i) {
    for (int32_t a = 0; a < D; ++a) {
      if (a) s.push_back(',');
      format_number<T>(y[i * D + a], s);
    }
    s.push_back('\n');
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return io_fail(BHTSNE_EIO, std::string("error: cannot create ") + path + ": " + std::strerror(errno));
  const bool ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
  const bool closed = std::fclose(f) == 0;
  if (!ok || !closed) return io_fail(BHTSNE_EIO, std::string("error: cannot write ") + path);
  return BHTSNE_OK;
}

}  // namespace

extern "C" {

const char* bhtsne_io_last_error(void) { return g_io_error.c_str(); }

int bhtsne_load_csv(const char* path, int32_t has_headers, const int64_t* skip, int64_t n_skip, int dtype, void* out,
                    int64_t* count, int64_t* records) {
  if (!path || !count || (n_skip > 0 && !skip) || n_skip < 0)
    return io_fail(BHTSNE_EINVAL, "error: invalid load_csv arguments.");
  if (dtype == BHTSNE_F32) return load_csv_impl<float>(path, has_headers, skip, n_skip, (float*)out, count, records);
  if (dtype == BHTSNE_F64) return load_csv_impl<double>(path, has_headers, skip, n_skip, (double*)out, count, records);
  return io_fail(BHTSNE_EINVAL, "error: dtype must be BHTSNE_F32 or BHTSNE_F64.");
}

int bhtsne_write_csv(const void* embedding, int64_t n, int32_t embed_dim, int dtype, const char* path) {
  if ((!embedding && n > 0) || !path || n < 0 || embed_dim < 1)
    return io_fail(BHTSNE_EINVAL, "error: invalid write_csv arguments.");
  if (dtype == BHTSNE_F32) return write_csv_impl<float>((const float*)embedding, n, embed_dim, path);
  if (dtype == BHTSNE_F64) return write_csv_impl<double>((const double*)embedding, n, embed_dim, path);
  return io_fail(BHTSNE_EINVAL, "error: dtype must be BHTSNE_F32 or BHTSNE_F64.");
}

}  // extern "C"

namespace bhg {
void set_host_error(const std::string& msg) { g_io_error = msg; }

int write_csv_file(const void* embedding, int64_t n, int32_t embed_dim, int dtype, const char* path) {
  return bhtsne_write_csv(embedding, n, embed_dim, dtype, path);
}
}  // namespace bhg
