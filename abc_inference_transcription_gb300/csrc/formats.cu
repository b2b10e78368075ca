// formats.cu — the reference's on-disk text files, written and read on the
// host: tab-delimited rows as DelimitedFiles.writedlm makes them.
//   particles_<model>.txt  one line per gene: the accepted 1-based particle
//                          indices in acceptance order, or a single 0
//                          (scripts/accepted_particles.jl:21-29; read back by
//                          scripts/posterior_kinetics.jl:56-60)
//   matrices               sets_<model>_<n>.txt (one theta row per particle,
//                          scripts/abc_simulation.jl:93-94), the statistics
//                          files s_pulse/s_chase (two rows per particle: means,
//                          Fano factors) and s_ratios/s_mean_corr/s_corr_mean
//                          (:47-60, read by scripts/compute_errors.jl:17-29),
//                          error_<model>.txt (one row of G errors per particle,
//                          :66-67), model_prob/l_bound/u_bound rows
//                          (scripts/model_probs.jl:54-61), posterior estimates
//                          (scripts/posterior_kinetics.jl:72-75).
// Floats are written in the shortest form that reads back to the same double,
// in Julia's spelling: fixed notation for 1e-4 <= |x| < 1e6 with a ".0" on
// integral values, otherwise an unpadded exponent ("1.0e-5", "1.234567e6"),
// NaN, Inf and -Inf.  Host code only; no GPU is involved.
#include <charconv>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/abcgpu.h"

namespace {

// Julia-style shortest decimal of x into buf; returns the length.  The digits
// are the shortest that read back to the same double; the notation follows
// Julia's float printing: with the decimal point pt places after the first
// digit's position (x = 0.d1d2... x 10^pt), fixed notation when -4 < pt <= 6
// (1e-4 <= |x| < 1e6: 100000.0, 0.0001, 0.00025, 123456.7), otherwise one
// digit, a point and an unpadded exponent (1.0e6, 1.234567e6, 1.0e-5).
int format_double(double x, char* buf) {
  if (std::isnan(x)) {
    std::memcpy(buf, "NaN", 3);
    return 3;
  }
  if (std::isinf(x)) {
    if (x > 0) {
      std::memcpy(buf, "Inf", 3);
      return 3;
    }
    std::memcpy(buf, "-Inf", 4);
    return 4;
  }
  char tmp[64];
  const auto res = std::to_chars(tmp, tmp + sizeof(tmp), x, std::chars_format::scientific);
  const int n = (int)(res.ptr - tmp);
  tmp[n] = '\0';  // to_chars does not terminate; atoi below needs it
  int i = 0, o = 0;
  if (tmp[i] == '-') {
    buf[o++] = '-';
    ++i;
  }
  char dig[32];
  int nd = 0;
  for (; i < n && tmp[i] != 'e'; ++i)
    if (tmp[i] != '.') dig[nd++] = tmp[i];
  int e10 = 0;
  if (i < n) e10 = std::atoi(tmp + i + 1);
  const int pt = e10 + 1;
  if (-4 < pt && pt <= 6) {
    if (pt <= 0) {
      buf[o++] = '0';
      buf[o++] = '.';
      for (int k = 0; k < -pt; ++k) buf[o++] = '0';
      for (int k = 0; k < nd; ++k) buf[o++] = dig[k];
    } else if (pt < nd) {
      for (int k = 0; k < pt; ++k) buf[o++] = dig[k];
      buf[o++] = '.';
      for (int k = pt; k < nd; ++k) buf[o++] = dig[k];
    } else {
      for (int k = 0; k < nd; ++k) buf[o++] = dig[k];
      for (int k = nd; k < pt; ++k) buf[o++] = '0';
      buf[o++] = '.';
      buf[o++] = '0';
    }
    return o;
  }
  buf[o++] = dig[0];
  buf[o++] = '.';
  if (nd == 1) buf[o++] = '0';
  for (int k = 1; k < nd; ++k) buf[o++] = dig[k];
  buf[o++] = 'e';
  const auto r2 = std::to_chars(buf + o, buf + o + 8, pt - 1);
  return (int)(r2.ptr - buf);
}

int format_int(long long v, char* buf) {
  const auto res = std::to_chars(buf, buf + 24, v);
  return (int)(res.ptr - buf);
}

// buffered writer: appends to a std::string, flushes in large blocks
struct Out {
  FILE* f = nullptr;
  std::string buf;
  bool ok = true;
  explicit Out(FILE* fp) : f(fp) { buf.reserve(1 << 22); }
  void put(const char* s, int n) {
    buf.append(s, (size_t)n);
    if (buf.size() >= (1u << 22)) flush();
  }
  void ch(char c) {
    buf.push_back(c);
    if (buf.size() >= (1u << 22)) flush();
  }
  void flush() {
    if (!buf.empty() && std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) ok = false;
    buf.clear();
  }
};

FILE* open_out(const char* path, int append) { return std::fopen(path, append ? "ab" : "wb"); }

}  // namespace

extern "C" {

int abc_write_particles(const char* path, int append, int64_t n_genes, const int64_t* gene_offsets,
                        const int64_t* particle_idx) {
  if (!path || n_genes < 0 || (n_genes > 0 && !gene_offsets)) return ABC_ERR_INVALID;
  if (n_genes > 0 && gene_offsets[n_genes] > gene_offsets[0] && !particle_idx) return ABC_ERR_INVALID;
  FILE* f = open_out(path, append);
  if (!f) return ABC_ERR_IO;
  Out out(f);
  char num[32];
  for (int64_t g = 0; g < n_genes; ++g) {
    const int64_t a = gene_offsets[g], b = gene_offsets[g + 1];
    if (b <= a) {
      out.ch('0');
    } else {
      for (int64_t i = a; i < b; ++i) {
        if (i > a) out.ch('\t');
        out.put(num, format_int(particle_idx[i], num));
      }
    }
    out.ch('\n');
  }
  out.flush();
  const bool ok = out.ok && std::fclose(f) == 0;
  return ok ? ABC_OK : ABC_ERR_IO;
}

int abc_write_matrix(const char* path, int append, int64_t rows, int64_t cols, const double* m, int64_t ld) {
  if (!path || rows < 0 || cols < 0 || (rows > 0 && cols > 0 && !m) || ld < cols) return ABC_ERR_INVALID;
  FILE* f = open_out(path, append);
  if (!f) return ABC_ERR_IO;
  Out out(f);
  char num[64];
  for (int64_t r = 0; r < rows; ++r) {
    const double* row = m + r * ld;
    for (int64_t c = 0; c < cols; ++c) {
      if (c) out.ch('\t');
      out.put(num, format_double(row[c], num));
    }
    out.ch('\n');
  }
  out.flush();
  const bool ok = out.ok && std::fclose(f) == 0;
  return ok ? ABC_OK : ABC_ERR_IO;
}

int abc_format_double(double x, char* buf, int buf_len) {
  if (!buf || buf_len < 32) return ABC_ERR_INVALID;
  const int n = format_double(x, buf);
  buf[n] = '\0';
  return n;
}

// particles file -> offsets and indices.  Call with particle_idx = NULL to
// get the sizes (*n_genes, *n_total: a line "0" is a gene without particles),
// then with buffers of those sizes.
int abc_read_particles(const char* path, int64_t* n_genes, int64_t* n_total, int64_t* gene_offsets,
                       int64_t* particle_idx) {
  if (!path || !n_genes || !n_total) return ABC_ERR_INVALID;
  FILE* f = std::fopen(path, "rb");
  if (!f) return ABC_ERR_IO;
  std::vector<char> data;
  {
    char chunk[1 << 16];
    size_t k;
    while ((k = std::fread(chunk, 1, sizeof(chunk), f)) > 0) data.insert(data.end(), chunk, chunk + k);
    std::fclose(f);
  }
  const bool fill = particle_idx != nullptr && gene_offsets != nullptr;
  int64_t g = 0, tot = 0;
  size_t i = 0;
  const size_t n = data.size();
  while (i < n) {
    // one line
    size_t e = i;
    while (e < n && data[e] != '\n') ++e;
    size_t le = e;
    if (le > i && data[le - 1] == '\r') --le;
    if (fill) gene_offsets[g] = tot;
    int64_t cnt = 0;
    bool zero_only = true;
    size_t p = i;
    while (p < le) {
      while (p < le && (data[p] == '\t' || data[p] == ' ')) ++p;
      if (p >= le) break;
      long long v = 0;
      const auto r = std::from_chars(data.data() + p, data.data() + le, v);
      if (r.ec != std::errc()) return ABC_ERR_IO;
      p = (size_t)(r.ptr - data.data());
      if (v != 0) zero_only = false;
      if (fill) particle_idx[tot + cnt] = v;
      ++cnt;
    }
    if (zero_only && cnt == 1) cnt = 0;  // the reference's "no particle" line
    tot += cnt;
    ++g;
    i = e + 1;
  }
  if (fill) gene_offsets[g] = tot;
  *n_genes = g;
  *n_total = tot;
  return ABC_OK;
}

}  // extern "C"
