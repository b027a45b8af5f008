// pimc_io.cpp -- files written from the engine's state: the paths and density
// tables of the reference's examples/tools/savetools.jl (CSV.jl output of its
// DataFrames) and a checksummed binary checkpoint.  Host code over the public
// C ABI; numbers are printed the way Julia prints a Float64.
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pimc.h"
#include "pimc_internal.h"

namespace {

// Julia's print of a Float64 (Base.Ryu.writeshortest, also used by CSV.jl):
// the shortest digits that round-trip, in fixed notation when the decimal
// point position pt (x = 0.d1d2... * 10^pt) satisfies -4 < pt <= 6, else as
// d.ddd e<exp> with at least one fractional digit ("1.0e-5", "1.234567e6").
std::string jfloat(double x) {
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "Inf" : "-Inf";
  if (x == 0.0) return std::signbit(x) ? "-0.0" : "0.0";
  char buf[64];
  auto r = std::to_chars(buf, buf + sizeof(buf), x, std::chars_format::scientific);
  std::string s(buf, r.ptr);
  std::string out;
  size_t i = 0;
  if (s[0] == '-') {
    out += '-';
    i = 1;
  }
  const size_t epos = s.find('e');
  std::string digits;
  for (size_t k = i; k < epos; ++k)
    if (s[k] != '.') digits += s[k];
  while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
  const int e10 = std::atoi(s.c_str() + epos + 1);
  const int pt = e10 + 1, nd = (int)digits.size();
  if (-4 < pt && pt <= 6) {
    if (pt <= 0) {
      out += "0.";
      out.append((size_t)(-pt), '0');
      out += digits;
    } else if (pt < nd) {
      out += digits.substr(0, (size_t)pt);
      out += '.';
      out += digits.substr((size_t)pt);
    } else {
      out += digits;
      out.append((size_t)(pt - nd), '0');
      out += ".0";
    }
  } else {
    out += digits[0];
    out += '.';
    out += nd > 1 ? digits.substr(1) : std::string("0");
    out += 'e';
    out += std::to_string(pt - 1);
  }
  return out;
}

int write_text(const char *path, const std::string &text) {
  FILE *f = std::fopen(path, "wb");
  if (!f) return pimc_fail(PIMC_EARG, std::string("cannot open ") + path + " for writing");
  const size_t n = std::fwrite(text.data(), 1, text.size(), f);
  const int closed = std::fclose(f);
  if (n != text.size() || closed != 0) return pimc_fail(PIMC_EARG, std::string("short write to ") + path);
  return PIMC_OK;
}

// FNV-1a, 64-bit
unsigned long long fnv1a(const unsigned char *p, size_t n) {
  unsigned long long h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

constexpr char kCkptMagic[8] = {'P', 'I', 'M', 'C', 'C', 'K', 'P', 'T'};

}  // namespace

extern "C" {

// paths_df + save_paths (examples/tools/savetools.jl:4-35): columns tau,
// "p<n> x"[, "p<n> y"] for every particle; M + 1 rows, tau = j beta / M, the
// last row the first bead of the next particle of the cycle
int pimc_write_paths_csv(void *handle, int chain, const char *path) {
  if (!handle || !path) return pimc_fail(PIMC_EARG, "null argument");
  pimc_params p;
  int rc = pimc_get_params(handle, chain, &p);
  if (rc) return rc;
  const int N = p.N, M = p.M, dim = p.dim;
  std::vector<double> x((size_t)dim * N * M);
  std::vector<int> nx((size_t)N);
  if ((rc = pimc_batch_get_beads(handle, chain, x.data()))) return rc;
  if ((rc = pimc_batch_get_next(handle, chain, nx.data()))) return rc;
  auto X = [&](int d, int n, int j) { return x[((size_t)d * N + n) * M + j]; };
  const double beta = 1.0 / p.T;
  std::string t = "tau";
  for (int n = 0; n < N; ++n) {
    t += ",p" + std::to_string(n + 1) + " x";
    if (dim == 2) t += ",p" + std::to_string(n + 1) + " y";
  }
  t += '\n';
  for (int j = 0; j <= M; ++j) {
    t += jfloat((double)j * beta / M);
    for (int n = 0; n < N; ++n)
      for (int d = 0; d < dim; ++d) {
        t += ',';
        t += jfloat(j < M ? X(d, n, j) : X(d, nx[n], 0));
      }
    t += '\n';
  }
  return write_text(path, t);
}

// density_df + save_density (savetools.jl:37-65): den = counts / (bin ndata),
// bin = 2L/nbins; first column pos = range(-L, L, length = nbins); in 2D the
// columns x1..x<nbins> hold den[:, k] (counts column-major, x index first)
int pimc_write_density_csv(const char *path, int dim, int nbins, double L, const double *counts,
                           unsigned long long ndata) {
  if (!path || !counts || nbins < 2 || (dim != 1 && dim != 2) || !(L > 0.0))
    return pimc_fail(PIMC_EARG, "density table needs a path, counts, dim 1 or 2, nbins >= 2, L > 0");
  const double bin = (2.0 * L) / nbins;
  const double norm = bin * (double)ndata;
  std::string t = "pos";
  if (dim == 1) {
    t += ",Density";
  } else {
    for (int k = 0; k < nbins; ++k) t += ",x" + std::to_string(k + 1);
  }
  t += '\n';
  for (int i = 0; i < nbins; ++i) {
    // -L + i 2L/(nbins-1), exact for the usual L as L*(2i - (nbins-1)) / (nbins-1)
    const double pos = (L * (double)(2 * i - (nbins - 1))) / (double)(nbins - 1);
    t += jfloat(pos);
    const int ncol = dim == 1 ? 1 : nbins;
    for (int k = 0; k < ncol; ++k) {
      t += ',';
      t += jfloat(counts[(size_t)i + (size_t)k * nbins] / norm);
    }
    t += '\n';
  }
  return write_text(path, t);
}

// checkpoint file: "PIMCCKPT", u64 ABI version, u64 state bytes, the state
// (pimc_get_state), u64 FNV-1a of the state
int pimc_save_checkpoint(void *handle, const char *path) {
  if (!handle || !path) return pimc_fail(PIMC_EARG, "null argument");
  size_t nb = 0;
  int rc = pimc_state_size(handle, &nb);
  if (rc) return rc;
  std::vector<unsigned char> blob(nb);
  if ((rc = pimc_get_state(handle, blob.data(), nb))) return rc;
  const unsigned long long ver = PIMC_ABI_VERSION, n64 = nb, sum = fnv1a(blob.data(), nb);
  std::string tmp = std::string(path) + ".tmp";
  FILE *f = std::fopen(tmp.c_str(), "wb");
  if (!f) return pimc_fail(PIMC_EARG, "cannot open " + tmp + " for writing");
  bool ok = std::fwrite(kCkptMagic, 1, 8, f) == 8 && std::fwrite(&ver, 8, 1, f) == 1 &&
            std::fwrite(&n64, 8, 1, f) == 1 && std::fwrite(blob.data(), 1, nb, f) == nb &&
            std::fwrite(&sum, 8, 1, f) == 1;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return pimc_fail(PIMC_EARG, std::string("cannot write checkpoint ") + path);
  }
  return PIMC_OK;
}

int pimc_load_checkpoint(void *handle, const char *path) {
  if (!handle || !path) return pimc_fail(PIMC_EARG, "null argument");
  size_t nb = 0;
  int rc = pimc_state_size(handle, &nb);
  if (rc) return rc;
  FILE *f = std::fopen(path, "rb");
  if (!f) return pimc_fail(PIMC_EARG, std::string("cannot open ") + path);
  char magic[8];
  unsigned long long ver = 0, n64 = 0, sum = 0;
  std::vector<unsigned char> blob;
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kCkptMagic, 8) == 0 &&
            std::fread(&ver, 8, 1, f) == 1 && std::fread(&n64, 8, 1, f) == 1;
  if (ok && (ver != PIMC_ABI_VERSION || n64 != nb)) {
    std::fclose(f);
    return pimc_fail(PIMC_ESTATE, std::string(path) + ": checkpoint of another version or handle shape");
  }
  if (ok) {
    blob.resize(nb);
    ok = std::fread(blob.data(), 1, nb, f) == nb && std::fread(&sum, 8, 1, f) == 1;
  }
  std::fclose(f);
  if (!ok) return pimc_fail(PIMC_ESTATE, std::string(path) + ": not a complete checkpoint file");
  if (fnv1a(blob.data(), nb) != sum) return pimc_fail(PIMC_ESTATE, std::string(path) + ": checksum mismatch");
  return pimc_set_state(handle, blob.data(), nb);
}

// Julia's print of a Float64, for callers that name files as the reference does
int pimc_format_float(double x, char *out, size_t cap) {
  const std::string s = jfloat(x);
  if (!out || cap < s.size() + 1) return pimc_fail(PIMC_EARG, "buffer too small");
  std::memcpy(out, s.c_str(), s.size() + 1);
  return PIMC_OK;
}

}  // extern "C"
