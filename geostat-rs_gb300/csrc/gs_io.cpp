// gs_io.cpp -- CSV input and output on either side of the kriging path
// (crates/geostat-cli/src/io_utils.rs).
//
// Reading follows the csv crate's default Reader (csv 1.4.0, the version
// the reference pins): the first record is the header, fields are separated
// by ',' and records by "\n", "\r" or "\r\n", a field may be quoted with '"'
// (a doubled quote inside stands for one), empty lines are skipped, and
// every record must have as many fields as the header.  A numeric field
// follows io_utils.rs parse_field: trimmed; empty, "na" or "nan" (any case)
// is missing; otherwise Rust's f64 grammar (optional sign, decimal digits
// with an optional fraction and exponent, or inf / infinity).  Rows with a
// missing or unparseable requested field are skipped and counted.
//
// Writing formats every number as Rust's `{}` does for f64: the shortest
// digits that round-trip, never in exponent form, "NaN", "inf", "-inf".
//
// Both directions split the work across host threads: the reader finds
// record boundaries in one quote-aware pass, then parses contiguous record
// ranges in parallel; the writer formats row ranges in parallel and writes
// them in order.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/geostat_gb300.h"
#include "gs_internal.h"

struct gs_csv_table {
  int ncols = 0;
  int64_t rows = 0;
  int64_t skipped = 0;
  std::vector<double> data;  // rows x ncols, row-major
};

namespace {

using gs::fail;

bool is_term(char c) { return c == '\n' || c == '\r'; }

// A record's fields: an unquoted field is a span of the input; a field that
// opens with a quote is decoded (doubled quotes become one, text after the
// closing quote joins the field) into `text`.
struct Field {
  const char* p;
  size_t n;
  int text;  // index into the record's decoded strings, or -1
};

struct Scanner {
  const char* buf;
  size_t len;

  // Walks one field from `pos`; decodes it when `dec` is set.
  size_t field_end(size_t pos, std::string* dec) const {
    if (pos < len && buf[pos] == '"') {
      ++pos;
      while (pos < len) {
        if (buf[pos] == '"') {
          if (pos + 1 < len && buf[pos + 1] == '"') {
            if (dec) dec->push_back('"');
            pos += 2;
            continue;
          }
          ++pos;
          break;
        }
        if (dec) dec->push_back(buf[pos]);
        ++pos;
      }
    }
    while (pos < len && buf[pos] != ',' && !is_term(buf[pos])) {
      if (dec) dec->push_back(buf[pos]);
      ++pos;
    }
    return pos;
  }

  // Skips blank lines; false at the end of the input.
  bool skip_blank(size_t& pos) const {
    while (pos < len && is_term(buf[pos])) ++pos;
    return pos < len;
  }

  // The record at `pos` (after blank lines) into `out`; pos moves past its
  // terminator ("\r\n", "\r" or "\n").
  bool next(size_t& pos, std::vector<Field>& out, std::vector<std::string>& texts) const {
    out.clear();
    texts.clear();
    if (!skip_blank(pos)) return false;
    for (;;) {
      const size_t start = pos;
      if (buf[pos] == '"') {
        texts.emplace_back();
        pos = field_end(pos, &texts.back());
        out.push_back(Field{nullptr, 0, (int)texts.size() - 1});
      } else {
        pos = field_end(pos, nullptr);
        out.push_back(Field{buf + start, pos - start, -1});
      }
      if (pos < len && buf[pos] == ',') {
        ++pos;
        if (pos >= len || is_term(buf[pos])) {  // a trailing empty field
          out.push_back(Field{buf + pos, 0, -1});
          break;
        }
        continue;
      }
      break;
    }
    if (pos < len && buf[pos] == '\r') {
      ++pos;
      if (pos < len && buf[pos] == '\n') ++pos;
    } else if (pos < len && buf[pos] == '\n') {
      ++pos;
    }
    return true;
  }

  // Record starts after `pos`, in one pass with the same field grammar.
  void record_starts(size_t pos, std::vector<size_t>& starts) const {
    while (skip_blank(pos)) {
      starts.push_back(pos);
      for (;;) {
        pos = field_end(pos, nullptr);
        if (pos < len && buf[pos] == ',') {
          ++pos;
          continue;
        }
        break;
      }
      if (pos < len && buf[pos] == '\r') {
        ++pos;
        if (pos < len && buf[pos] == '\n') ++pos;
      } else if (pos < len && buf[pos] == '\n') {
        ++pos;
      }
    }
  }
};

bool ieq(const char* a, size_t n, const char* lit) {
  const size_t m = std::strlen(lit);
  if (n != m) return false;
  for (size_t i = 0; i < n; ++i) {
    char c = a[i];
    if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
    if (c != lit[i]) return false;
  }
  return true;
}

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }

// io_utils.rs parse_field: false = missing or unparseable.
bool parse_number(const char* p, size_t n, double* out) {
  while (n > 0 && is_space(*p)) {
    ++p;
    --n;
  }
  while (n > 0 && is_space(p[n - 1])) --n;
  if (n == 0 || ieq(p, n, "na") || ieq(p, n, "nan")) return false;
  bool neg = false;
  const char* s = p;
  size_t m = n;
  if (*s == '+' || *s == '-') {
    neg = *s == '-';
    ++s;
    --m;
  }
  if (m == 0) return false;
  if (ieq(s, m, "inf") || ieq(s, m, "infinity")) {
    *out = neg ? -INFINITY : INFINITY;
    return true;
  }
  // Rust's decimal grammar: digits [. digits] [(e|E) [sign] digits], with
  // at least one digit before or after the point
  size_t i = 0, mant = 0;
  while (i < m && s[i] >= '0' && s[i] <= '9') ++i, ++mant;
  if (i < m && s[i] == '.') {
    ++i;
    while (i < m && s[i] >= '0' && s[i] <= '9') ++i, ++mant;
  }
  if (mant == 0) return false;
  if (i < m && (s[i] == 'e' || s[i] == 'E')) {
    ++i;
    if (i < m && (s[i] == '+' || s[i] == '-')) ++i;
    size_t ed = 0;
    while (i < m && s[i] >= '0' && s[i] <= '9') ++i, ++ed;
    if (ed == 0) return false;
  }
  if (i != m) return false;
  double v = 0.0;
  auto r = std::from_chars(s, s + m, v, std::chars_format::general);
  if (r.ec == std::errc::result_out_of_range || r.ptr != s + m) {
    std::string tmp(s, m);  // overflow to inf / underflow to zero, correctly rounded
    v = std::strtod(tmp.c_str(), nullptr);
  } else if (r.ec != std::errc()) {
    return false;
  }
  *out = neg ? -v : v;
  return true;
}

int hw_threads(int requested) {
  if (requested > 0) return requested;
  const unsigned h = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(h, 64u));
}

// Rust's Display for f64 into `buf` (at least 400 bytes); returns the length.
size_t format_f64(double v, char* buf) {
  if (std::isnan(v)) {
    std::memcpy(buf, "NaN", 3);
    return 3;
  }
  if (std::isinf(v)) {
    if (v < 0) {
      std::memcpy(buf, "-inf", 4);
      return 4;
    }
    std::memcpy(buf, "inf", 3);
    return 3;
  }
  // the shortest round-trip digits (scientific form), laid out without an
  // exponent and padded with zeros as Rust does
  char sci[64];
  auto r = std::to_chars(sci, sci + sizeof(sci) - 1, v, std::chars_format::scientific);
  *r.ptr = '\0';
  const char* p = sci;
  const char* end = r.ptr;
  size_t k = 0;
  if (*p == '-') {
    buf[k++] = '-';
    ++p;
  }
  char dig[32];
  int nd = 0;
  const char* q = p;
  for (; q < end && *q != 'e'; ++q)
    if (*q != '.') dig[nd++] = *q;
  const int e10 = std::atoi(q + 1);  // value = 0.d1d2.. x 10^(e10 + 1)
  while (nd > 1 && dig[nd - 1] == '0') --nd;
  const int point = e10 + 1;  // digits before the decimal point
  if (point <= 0) {
    buf[k++] = '0';
    if (!(nd == 1 && dig[0] == '0')) {
      buf[k++] = '.';
      for (int i = 0; i < -point; ++i) buf[k++] = '0';
      for (int i = 0; i < nd; ++i) buf[k++] = dig[i];
    }
  } else if (point >= nd) {
    for (int i = 0; i < nd; ++i) buf[k++] = dig[i];
    for (int i = nd; i < point; ++i) buf[k++] = '0';
  } else {
    for (int i = 0; i < point; ++i) buf[k++] = dig[i];
    buf[k++] = '.';
    for (int i = point; i < nd; ++i) buf[k++] = dig[i];
  }
  return k;
}

}  // namespace

extern "C" {

int gs_csv_read(const char* path, const char* const* cols, int ncols, int nthreads,
                gs_csv_table** out) {
  if (!path || !out || ncols <= 0 || !cols) return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  *out = nullptr;
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return fail(GS_ERR_IO, std::string("cannot open input file ") + path);
  std::string buf;
  {
    std::fseek(fp, 0, SEEK_END);
    const long sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    buf.resize(sz > 0 ? (size_t)sz : 0);
    const size_t got = sz > 0 ? std::fread(&buf[0], 1, (size_t)sz, fp) : 0;
    std::fclose(fp);
    if (got != buf.size()) return fail(GS_ERR_IO, std::string("cannot read input file ") + path);
  }
  Scanner sc{buf.data(), buf.size()};
  size_t pos = 0;
  std::vector<Field> fields;
  std::vector<std::string> texts;
  if (buf.size() >= 3 && (unsigned char)buf[0] == 0xEF && (unsigned char)buf[1] == 0xBB &&
      (unsigned char)buf[2] == 0xBF)
    pos = 3;  // a UTF-8 byte-order mark before the header
  if (!sc.next(pos, fields, texts)) return fail(GS_ERR_IO, "cannot read CSV header");
  std::vector<std::string> header;
  for (const Field& f : fields) header.push_back(f.text >= 0 ? texts[f.text] : std::string(f.p, f.n));
  std::vector<int> idx(ncols);
  for (int c = 0; c < ncols; ++c) {
    const std::string name = cols[c] ? cols[c] : "";
    auto it = std::find(header.begin(), header.end(), name);
    if (it == header.end()) {
      std::string avail;
      for (size_t h = 0; h < header.size(); ++h) avail += (h ? ", " : "") + header[h];
      return fail(GS_ERR_INVALID_PARAMETER,
                  "column '" + name + "' not found; available columns: " + avail);
    }
    idx[c] = (int)(it - header.begin());
  }
  const size_t nfields = header.size();
  // record starts, one pass
  std::vector<size_t> starts;
  sc.record_starts(pos, starts);
  const int64_t nrec = (int64_t)starts.size();
  const int T = (int)std::max<int64_t>(1, std::min<int64_t>(hw_threads(nthreads), (nrec + 4095) / 4096));
  struct Part {
    std::vector<double> data;
    int64_t skipped = 0;
    int64_t bad_row = -1;
    size_t bad_fields = 0;
  };
  std::vector<Part> parts(T);
  auto work = [&](int t) {
    const int64_t lo = nrec * t / T, hi = nrec * (t + 1) / T;
    Part& P = parts[t];
    std::vector<Field> fs;
    std::vector<std::string> tx;
    std::vector<double> row(ncols);
    for (int64_t r = lo; r < hi; ++r) {
      size_t p = starts[r];
      sc.next(p, fs, tx);
      if (fs.size() != nfields) {
        P.bad_row = r;
        P.bad_fields = fs.size();
        return;
      }
      bool ok = true;
      for (int c = 0; c < ncols && ok; ++c) {
        const Field& f = fs[idx[c]];
        if (f.text >= 0) {
          const std::string& s = tx[f.text];
          ok = parse_number(s.data(), s.size(), &row[c]);
        } else {
          ok = parse_number(f.p, f.n, &row[c]);
        }
      }
      if (!ok) {
        ++P.skipped;
        continue;
      }
      P.data.insert(P.data.end(), row.begin(), row.end());
    }
  };
  if (T == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t) th.emplace_back(work, t);
    for (auto& x : th) x.join();
  }
  auto* tab = new gs_csv_table;
  tab->ncols = ncols;
  for (const Part& P : parts) {
    if (P.bad_row >= 0) {
      delete tab;
      return fail(GS_ERR_IO, "cannot parse CSV row " + std::to_string(P.bad_row + 2) + ": found " +
                                 std::to_string(P.bad_fields) + " fields, the header has " +
                                 std::to_string(nfields));
    }
  }
  size_t total = 0;
  for (const Part& P : parts) total += P.data.size();
  tab->data.reserve(total);
  for (const Part& P : parts) {
    tab->data.insert(tab->data.end(), P.data.begin(), P.data.end());
    tab->skipped += P.skipped;
  }
  tab->rows = (int64_t)(tab->data.size() / ncols);
  *out = tab;
  return GS_OK;
}

int gs_csv_table_info(const gs_csv_table* t, int64_t* rows, int64_t* skipped) {
  if (!t) return fail(GS_ERR_INVALID_PARAMETER, "null table");
  if (rows) *rows = t->rows;
  if (skipped) *skipped = t->skipped;
  return GS_OK;
}

int gs_csv_table_copy(const gs_csv_table* t, double* out) {
  if (!t || (!out && t->rows > 0)) return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  if (!t->data.empty()) std::memcpy(out, t->data.data(), t->data.size() * sizeof(double));
  return GS_OK;
}

void gs_csv_table_destroy(gs_csv_table* t) { delete t; }

int gs_csv_write(const char* path, const char* header, int ncols, const double* const* columns,
                 int64_t nrows, int nthreads) {
  if (!path || !header || ncols <= 0 || !columns || nrows < 0)
    return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  for (int c = 0; c < ncols; ++c)
    if (!columns[c] && nrows > 0) return fail(GS_ERR_INVALID_PARAMETER, "null column");
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return fail(GS_ERR_IO, std::string("cannot create output file ") + path);
  const int T = (int)std::max<int64_t>(1, std::min<int64_t>(hw_threads(nthreads), (nrows + 65535) / 65536));
  // blocks of rows formatted in parallel, written in order
  const int64_t block = 1 << 16;
  const int64_t nblocks = (nrows + block - 1) / block;
  std::vector<std::string> out((size_t)std::max<int64_t>(nblocks, 1));
  bool ok = std::fputs(header, fp) >= 0 && std::fputc('\n', fp) != EOF;
  for (int64_t b0 = 0; b0 < nblocks && ok; b0 += T) {
    const int64_t b1 = std::min(nblocks, b0 + T);
    auto work = [&](int64_t b) {
      std::string& s = out[(size_t)(b - b0)];
      s.clear();
      char num[400];
      const int64_t lo = b * block, hi = std::min(nrows, lo + block);
      for (int64_t r = lo; r < hi; ++r) {
        for (int c = 0; c < ncols; ++c) {
          if (c) s.push_back(',');
          const size_t k = format_f64(columns[c][r], num);
          s.append(num, k);
        }
        s.push_back('\n');
      }
    };
    if (b1 - b0 == 1) {
      work(b0);
    } else {
      std::vector<std::thread> th;
      for (int64_t b = b0; b < b1; ++b) th.emplace_back(work, b);
      for (auto& x : th) x.join();
    }
    for (int64_t b = b0; b < b1 && ok; ++b) {
      const std::string& s = out[(size_t)(b - b0)];
      ok = std::fwrite(s.data(), 1, s.size(), fp) == s.size();
    }
  }
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) return fail(GS_ERR_IO, std::string("cannot write output file ") + path);
  return GS_OK;
}

}  // extern "C"
