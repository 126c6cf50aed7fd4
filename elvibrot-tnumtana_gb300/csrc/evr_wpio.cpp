// evr_wpio.cpp -- wave-packet files in the reference's save formats (host only).
//
// A Fortran host and this library exchange packets (start vectors, restart files, the
// levels' eigenvectors) through the files the reference writes and reads:
//   sub_save_psi / Write_header_saveFile_psi / Write_Psi_nDBasis
//     (Source_ElVibRot/sub_WP/sub_module_psi_io.f90:365-424, 1441-1778)
//   ecri_psiBasisRepnotall_nD (:783-917)                        -- sparse packets
//   sub_read_psi0 / Read_header_saveFile_psi / Read_list_nDindBasis1_TO_nDindBasis2 /
//   Read_psi_nDBasis / lect_psiBasisRepnotall_nD (:55-263, 1294-1439, 1143-1292, 920-1141,
//     563-780)
// Every basis function is identified by its tuple (n_1..n_D, i_h, i_e), 1-based, which
// the reference gets from Rec_ndim_index (sub_module_basis.f90:3156).  Here n comes from
// the packed table, i_h = 1 and i_e = electronic state + 1, and the packed index of
// function k in state a is a*Np + k (i_bhe = i_b + ((i_h-1) + (i_e-1)*nb_bi)*nb_ba).
// Reading maps each tuple of the file onto this basis (calc_InD_FROM_ndim_index), so a
// file written on a smaller or larger basis fills the common functions, leaves the others
// at zero and drops (and counts) the functions this basis does not hold.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "evr_internal.h"

namespace {

using evr::HostProblem;
using evr::set_error;

// Lookup of a packed function from its 1-based tuple.
struct TupleIndex {
  int D = 0;
  std::vector<int> nmax;  // largest n per mode in the packed set
  std::unordered_map<uint64_t, int64_t> rank;

  explicit TupleIndex(const HostProblem& P) : D(P.D), nmax(P.D, 1) {
    for (int64_t k = 0; k < P.Np; ++k)
      for (int i = 0; i < D; ++i) nmax[i] = std::max(nmax[i], P.packed[(size_t)k * D + i]);
    rank.reserve((size_t)P.Np * 2);
    for (int64_t k = 0; k < P.Np; ++k) rank[key(&P.packed[(size_t)k * D])] = k;
  }
  uint64_t key(const int* n) const {
    uint64_t k = 0;
    for (int i = 0; i < D; ++i) k = k * (uint64_t)(nmax[i] + 1) + (uint64_t)n[i];
    return k;
  }
  // packed index of n, or -1 when n is not in this basis
  int64_t find(const int* n) const {
    for (int i = 0; i < D; ++i)
      if (n[i] < 1 || n[i] > nmax[i]) return -1;
    auto it = rank.find(key(n));
    return it == rank.end() ? -1 : it->second;
  }
};

// ---------------------------------------------------------------- writing

// gfortran-style list-directed real: 17 significant digits, three-digit exponent.
void put_real(std::string& s, double v) {
  char b[48];
  snprintf(b, sizeof b, " %24.16E", v);
  s += b;
}

struct Out {
  FILE* f = nullptr;
  ~Out() {
    if (f) fclose(f);
  }
};

bool put_record(FILE* f, const void* p, size_t n) {
  const int32_t m = (int32_t)n;
  return fwrite(&m, 4, 1, f) == 1 && (n == 0 || fwrite(p, 1, n, f) == n) && fwrite(&m, 4, 1, f) == 1;
}

double val(const double* psi, int64_t ld, int cplx, int j, int64_t k, int part) {
  return cplx ? psi[2 * (k + ld * j) + part] : psi[k + ld * j];
}

// ---------------------------------------------------------------- reading

// Fortran numeric token -> double: accepts D/Q exponents and the exponent without a
// letter that some compilers write for three-digit exponents (1.0+100).
bool parse_real(const std::string& t, double* out) {
  if (t.empty()) return false;
  {  // common case: a C-style number, read in place
    char* end = nullptr;
    *out = strtod(t.c_str(), &end);
    if (end && *end == '\0' && end != t.c_str()) return true;
  }
  std::string u;
  u.reserve(t.size() + 1);
  for (size_t i = 0; i < t.size(); ++i) {
    char ch = t[i];
    if (ch == 'd' || ch == 'D' || ch == 'q' || ch == 'Q') ch = 'E';
    if ((ch == '+' || ch == '-') && i > 0 && (isdigit((unsigned char)t[i - 1]) || t[i - 1] == '.')) u += 'E';
    u += ch;
  }
  char* end = nullptr;
  *out = strtod(u.c_str(), &end);
  return end && *end == '\0' && end != u.c_str();
}

bool parse_int(const std::string& t, long long* out) {
  if (t.empty()) return false;
  char* end = nullptr;
  *out = strtoll(t.c_str(), &end, 10);
  return end && *end == '\0';
}

// Splits a line into list-directed items (blanks and commas separate; a parenthesised
// complex constant stays one item).
std::vector<std::string> items_of(const std::string& line) {
  std::vector<std::string> v;
  const size_t n = line.size();
  size_t i = 0;
  while (i < n) {
    while (i < n && (isspace((unsigned char)line[i]) || line[i] == ',')) ++i;
    if (i >= n) break;
    size_t j = i;
    int depth = 0;
    for (; j < n; ++j) {
      const char ch = line[j];
      if (ch == '(') ++depth;
      else if (ch == ')') --depth;
      else if (depth == 0 && (isspace((unsigned char)ch) || ch == ',')) break;
    }
    v.push_back(line.substr(i, j - i));
    i = j;
  }
  return v;
}

// One value item: "x", "(re,im)", with an optional repeat count "r*".
bool parse_value_item(const std::string& it0, int cplx, long long* rep, double* re, double* im) {
  std::string it = it0;
  *rep = 1;
  const size_t star = it.find('*');
  if (star != std::string::npos) {
    if (!parse_int(it.substr(0, star), rep) || *rep < 1) return false;
    it = it.substr(star + 1);
  }
  *im = 0.0;
  if (cplx) {
    if (it.size() < 5 || it.front() != '(' || it.back() != ')') return false;
    std::string in = it.substr(1, it.size() - 2);
    const size_t comma = in.find(',');
    if (comma == std::string::npos) return false;
    auto trim = [](std::string s) {
      size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
      return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    };
    return parse_real(trim(in.substr(0, comma)), re) && parse_real(trim(in.substr(comma + 1)), im);
  }
  return parse_real(it, re);
}

// An index/value line "n_1 .. n_D i_h i_e a [b]" (list-directed: extra items are ignored).
bool parse_entry(const std::vector<std::string>& it, int D, int cplx, int* n, double* a, double* b) {
  const size_t need = (size_t)D + 2 + (cplx ? 2 : 1);
  if (it.size() < need) return false;
  for (int i = 0; i < D + 2; ++i) {
    long long v;
    if (!parse_int(it[i], &v) || v < -2147483647LL || v > 2147483647LL) return false;
    n[i] = (int)v;
  }
  *b = 0.0;
  if (!parse_real(it[D + 2], a)) return false;
  if (cplx && !parse_real(it[D + 3], b)) return false;
  return true;
}

// Destination of one file entry: packed row, or -1 when this basis does not hold it.
int64_t dest_row(const TupleIndex& T, const HostProblem& P, const int* n) {
  const int ih = n[P.D], ie = n[P.D + 1];
  if (ih != 1 || ie < 1 || ie > P.nb0) return -1;
  const int64_t k = T.find(n);
  return k < 0 ? -1 : (int64_t)(ie - 1) * P.Np + k;
}

struct Reader {
  evr_ctx* c;
  const HostProblem& P;
  TupleIndex T;
  double* psi;
  int64_t ld;
  int npsi_max, cplx;
  int stored = 0;
  int64_t dropped = 0;

  Reader(evr_ctx* c_, double* psi_, int64_t ld_, int npsi_max_, int cplx_)
      : c(c_), P(c_->hp), T(c_->hp), psi(psi_), ld(ld_), npsi_max(npsi_max_), cplx(cplx_) {}

  void clear(int j) {
    const int64_t N = P.Np * P.nb0, w = cplx ? 2 : 1;
    std::fill(psi + w * ld * j, psi + w * ld * j + w * N, 0.0);
  }
  void put(int j, int64_t row, double a, double b) {
    if (cplx) {
      psi[2 * (row + ld * j)] = a;
      psi[2 * (row + ld * j) + 1] = b;
    } else {
      psi[row + ld * j] = a;
    }
  }

  // Formatted files: nb_psi (and nb_tot) header lines, a namelist header, or no header.
  int formatted(const std::vector<std::string>& lines) {
    size_t li = 0;
    while (li < lines.size() && lines[li].find_first_not_of(" \t\r") == std::string::npos) ++li;
    if (li == lines.size()) return set_error(c, EVR_EINVAL, "evr_psi_read: empty file");
    const std::string& head = lines[li];
    const size_t h0 = head.find_first_not_of(" \t");
    if (head[h0] == '&' || head[h0] == '$') return namelist_v1(lines, li);
    std::vector<std::string> it = items_of(head);
    long long a = 0, b = 0;
    if (it.size() == 1 && parse_int(it[0], &a)) return sparse(lines, li + 1, a);
    if (it.size() == 2 && parse_int(it[0], &a) && parse_int(it[1], &b)) return positional_v0(lines, li + 1, a, b);
    return sparse(lines, li, -1);  // packets without a header (the packets of an input file)
  }

  // lect_psiBasisRepnotall_nD: each packet is a list of entries ended by a line that is
  // not an entry ("end wp ..."); entries are placed by their tuple.
  int sparse(const std::vector<std::string>& lines, size_t li, long long nb_psi) {
    std::vector<int> n(P.D + 2);
    int packet = 0;
    bool open = false;
    for (; li < lines.size(); ++li) {
      if (nb_psi >= 0 && packet >= nb_psi) break;
      if (packet >= npsi_max) break;
      std::vector<std::string> it = items_of(lines[li]);
      if (it.empty()) continue;
      double x, y;
      if (!parse_entry(it, P.D, cplx, n.data(), &x, &y)) {
        if (!open) clear(packet);
        open = false;
        ++packet;
        continue;
      }
      if (!open) clear(packet), open = true;
      const int64_t r = dest_row(T, P, n.data());
      if (r < 0) ++dropped;
      else put(packet, r, x, y);
    }
    if (open) ++packet;
    stored = std::min(packet, npsi_max);
    if (nb_psi > 0 && stored < std::min<long long>(nb_psi, npsi_max))
      return set_error(c, EVR_EINVAL, "evr_psi_read: file ends after " + std::to_string(stored) + " of " +
                                          std::to_string(nb_psi) + " packets");
    return EVR_OK;
  }

  // Version 0 with "nb_psi nb_tot": every packet lists all nb_tot entries in the same
  // order, then an "end wp" line; the first packet's tuples give the list
  // (Read_list_nDindBasis1_TO_nDindBasis2 version 0) and every packet is read by position.
  int positional_v0(const std::vector<std::string>& lines, size_t li, long long nb_psi, long long nb_tot) {
    if (nb_psi < 0 || nb_tot < 1) return set_error(c, EVR_EINVAL, "evr_psi_read: bad header (nb_psi nb_tot)");
    std::vector<int64_t> list;
    std::vector<int> n(P.D + 2);
    for (long long p = 0; p < nb_psi && p < npsi_max; ++p) {
      clear((int)p);
      for (long long e = 0; e < nb_tot; ++e, ++li) {
        while (li < lines.size() && lines[li].find_first_not_of(" \t\r") == std::string::npos) ++li;
        double x, y;
        if (li >= lines.size() || !parse_entry(items_of(lines[li]), P.D, cplx, n.data(), &x, &y))
          return set_error(c, EVR_EINVAL, "evr_psi_read: packet " + std::to_string(p + 1) + " has fewer than nb_tot = " +
                                              std::to_string(nb_tot) + " entries (or a line that is not n_1..n_D i_h i_e value)");
        if (p == 0) list.push_back(dest_row(T, P, n.data()));
        const int64_t r = list[(size_t)e];
        if (r < 0) ++dropped;
        else put((int)p, r, x, y);
      }
      while (li < lines.size() && lines[li].find_first_not_of(" \t\r") == std::string::npos) ++li;
      if (li >= lines.size() || lines[li].find("end") == std::string::npos)
        return set_error(c, EVR_EINVAL, "evr_psi_read: packet " + std::to_string(p + 1) + " is not followed by its 'end wp' line");
      ++li;
      ++stored;
    }
    if (stored < std::min<long long>(nb_psi, npsi_max))
      return set_error(c, EVR_EINVAL, "evr_psi_read: fewer packets than the header's nb_psi");
    return EVR_OK;
  }

  // Version 1 with the headerFile namelist: the list of nb_tot tuples, then each packet
  // as one list-directed record of nb_tot values.
  int namelist_v1(const std::vector<std::string>& lines, size_t li) {
    std::string nl;
    bool closed = false;
    for (; li < lines.size() && !closed; ++li) {
      const std::string& L = lines[li];
      for (size_t i = 0; i < L.size(); ++i) {
        if (L[i] == '/') { closed = true; break; }
        nl += (char)toupper((unsigned char)L[i]);
      }
      if (!closed) nl += ' ';
      size_t e = nl.find("&END");
      if (e == std::string::npos) e = nl.find("$END");
      if (e != std::string::npos && e > 0) { nl.resize(e); closed = true; }
    }
    if (!closed) return set_error(c, EVR_EINVAL, "evr_psi_read: headerFile namelist is not closed");
    const size_t g = nl.find("HEADERFILE");
    if (g == std::string::npos) return set_error(c, EVR_EINVAL, "evr_psi_read: namelist is not headerFile");
    long long version = 0, nb_psi = 0, nb_tot = 0;  // Version_File defaults to FilePsiVersion = 0
    std::string body = nl.substr(g + 10);
    for (char& ch : body)
      if (ch == '=' || ch == ',') ch = ' ';
    std::vector<std::string> it = items_of(body);
    for (size_t i = 0; i + 1 < it.size(); i += 2) {
      long long v;
      if (!parse_int(it[i + 1], &v)) return set_error(c, EVR_EINVAL, "evr_psi_read: headerFile value of " + it[i]);
      if (it[i] == "VERSION_FILE") version = v;
      else if (it[i] == "NB_PSI") nb_psi = v;
      else if (it[i] == "NB_TOT") nb_tot = v;
      else return set_error(c, EVR_EINVAL, "evr_psi_read: unknown headerFile item " + it[i]);
    }
    if (it.size() % 2) return set_error(c, EVR_EINVAL, "evr_psi_read: malformed headerFile namelist");
    if (version != 1) return set_error(c, EVR_EINVAL, "evr_psi_read: a headerFile namelist with Version_File /= 1");
    if (nb_psi < 0 || nb_tot < 1) return set_error(c, EVR_EINVAL, "evr_psi_read: bad nb_psi / nb_tot in headerFile");
    std::vector<int64_t> list;
    list.reserve((size_t)nb_tot);
    std::vector<int> n(P.D + 2);
    for (long long e = 0; e < nb_tot; ++e, ++li) {
      while (li < lines.size() && lines[li].find_first_not_of(" \t\r") == std::string::npos) ++li;
      if (li >= lines.size()) return set_error(c, EVR_EINVAL, "evr_psi_read: index list shorter than nb_tot");
      std::vector<std::string> iv = items_of(lines[li]);
      if (iv.size() < (size_t)P.D + 2) return set_error(c, EVR_EINVAL, "evr_psi_read: index line with fewer than D+2 integers");
      for (int i = 0; i < P.D + 2; ++i) {
        long long v;
        if (!parse_int(iv[i], &v) || v < -2147483647LL || v > 2147483647LL)
          return set_error(c, EVR_EINVAL, "evr_psi_read: index list line " + std::to_string(e + 1));
        n[i] = (int)v;
      }
      list.push_back(dest_row(T, P, n.data()));
    }
    // values: a stream of items over the remaining lines
    long long e = 0, p = 0, rep = 0;
    double x = 0, y = 0;
    if (nb_psi > 0 && npsi_max > 0) clear(0);
    for (; li < lines.size() && p < nb_psi && p < npsi_max; ++li) {
      for (const std::string& item : items_of(lines[li])) {
        if (!parse_value_item(item, cplx, &rep, &x, &y))
          return set_error(c, EVR_EINVAL, std::string("evr_psi_read: value '") + item + "' is not a " +
                                              (cplx ? "complex (re,im)" : "real") + " constant");
        for (long long r = 0; r < rep && p < nb_psi && p < npsi_max; ++r) {
          const int64_t row = list[(size_t)e];
          if (row < 0) ++dropped;
          else put((int)p, row, x, y);
          if (++e == nb_tot) {
            e = 0;
            ++p;
            ++stored;
            if (p < nb_psi && p < npsi_max) clear((int)p);
          }
        }
        if (p >= nb_psi || p >= npsi_max) break;
      }
    }
    if (stored < std::min<long long>(nb_psi, npsi_max))
      return set_error(c, EVR_EINVAL, "evr_psi_read: file ends inside packet " + std::to_string(stored + 1));
    return EVR_OK;
  }

  // Unformatted (Fortran sequential records with 4-byte length markers): 'X', nb_psi,
  // nb_tot, Version_File = 1, 'X', nb_tot index records, one value record per packet.
  int unformatted(const std::vector<unsigned char>& buf) {
    size_t pos = 0;
    auto rec = [&](const unsigned char** p, size_t* n) {
      if (pos + 4 > buf.size()) return false;
      int32_t m1, m2;
      memcpy(&m1, &buf[pos], 4);
      if (m1 < 0 || pos + 8 + (size_t)m1 > buf.size()) return false;
      memcpy(&m2, &buf[pos + 4 + (size_t)m1], 4);
      if (m1 != m2) return false;
      *p = &buf[pos + 4];
      *n = (size_t)m1;
      pos += 8 + (size_t)m1;
      return true;
    };
    const unsigned char* p;
    size_t n;
    auto get_int = [&](long long* v, size_t* width) {
      if (!rec(&p, &n) || (n != 4 && n != 8)) return false;
      *width = n;
      if (n == 4) {
        int32_t t;
        memcpy(&t, p, 4);
        *v = t;
      } else {
        int64_t t;
        memcpy(&t, p, 8);
        *v = t;
      }
      return true;
    };
    long long nb_psi, nb_tot, version;
    size_t ik = 4, w2, w3;
    if (!rec(&p, &n) || n != 1 || p[0] != 'X' || !get_int(&nb_psi, &ik) || !get_int(&nb_tot, &w2) ||
        !get_int(&version, &w3) || !rec(&p, &n) || n != 1 || p[0] != 'X')
      return set_error(c, EVR_EINVAL, "evr_psi_read: unformatted header ('X', nb_psi, nb_tot, version, 'X') not found");
    if (version != 1) return set_error(c, EVR_EINVAL, "evr_psi_read: unformatted file with Version_File /= 1");
    if (nb_psi < 0 || nb_tot < 1) return set_error(c, EVR_EINVAL, "evr_psi_read: bad nb_psi / nb_tot");
    std::vector<int64_t> list((size_t)nb_tot);
    std::vector<int> nd(P.D + 2);
    for (long long e = 0; e < nb_tot; ++e) {
      if (!rec(&p, &n) || n != (size_t)(P.D + 2) * ik)
        return set_error(c, EVR_EINVAL, "evr_psi_read: index record " + std::to_string(e + 1) + " does not hold D+2 integers");
      for (int i = 0; i < P.D + 2; ++i) {
        if (ik == 4) {
          int32_t t;
          memcpy(&t, p + 4 * i, 4);
          nd[i] = t;
        } else {
          int64_t t;
          memcpy(&t, p + 8 * i, 8);
          nd[i] = (t < -2147483647LL || t > 2147483647LL) ? 0 : (int)t;
        }
      }
      list[(size_t)e] = dest_row(T, P, nd.data());
    }
    const size_t need = (size_t)nb_tot * (cplx ? 16 : 8);
    for (long long q = 0; q < nb_psi && q < npsi_max; ++q) {
      if (!rec(&p, &n)) return set_error(c, EVR_EINVAL, "evr_psi_read: file ends before packet " + std::to_string(q + 1));
      if (n != need)
        return set_error(c, EVR_EINVAL, "evr_psi_read: packet record of " + std::to_string(n) + " bytes, expected " +
                                            std::to_string(need) + (cplx ? " (complex)" : " (real)"));
      clear((int)q);
      for (long long e = 0; e < nb_tot; ++e) {
        double x, y = 0.0;
        memcpy(&x, p + (cplx ? 16 : 8) * e, 8);
        if (cplx) memcpy(&y, p + 16 * e + 8, 8);
        const int64_t row = list[(size_t)e];
        if (row < 0) ++dropped;
        else put((int)q, row, x, y);
      }
      ++stored;
    }
    return EVR_OK;
  }
};

int check_ctx(evr_ctx* c, const char* who) {
  if (!c) return EVR_EINVAL;
  if (c->batch) return set_error(c, EVR_EINVAL, std::string(who) + ": not for batched contexts");
  return EVR_OK;
}

}  // namespace

extern "C" int evr_psi_write(evr_ctx* c, const char* path, int format, const double* psi, int64_t ld, int npsi,
                             int cplx, double epsi) {
  if (int rc = check_ctx(c, "evr_psi_write")) return rc;
  const HostProblem& P = c->hp;
  const int64_t N = P.Np * P.nb0;
  if (!path || !psi || npsi < 0 || ld < N || (cplx != 0 && cplx != 1) || format < EVR_WP_FORMATTED_V0 ||
      format > EVR_WP_SPARSE || !(epsi >= 0.0))
    return set_error(c, EVR_EINVAL, "evr_psi_write: null pointer, ld < N, npsi < 0, bad format, cplx or epsi");
  if (format == EVR_WP_UNFORMATTED_V1 && (double)N * (cplx ? 16 : 8) > 2147483647.0)
    return set_error(c, EVR_EINVAL, "evr_psi_write: a packet record exceeds 2 GiB (4-byte record markers)");
  Out o;
  o.f = fopen(path, format == EVR_WP_UNFORMATTED_V1 ? "wb" : "w");
  if (!o.f) return set_error(c, EVR_EINVAL, std::string("evr_psi_write: cannot open ") + path);
  const int D = P.D;
  std::string s;
  auto flush = [&]() {
    bool ok = s.empty() || fwrite(s.data(), 1, s.size(), o.f) == s.size();
    s.clear();
    return ok;
  };
  // the text of each row's tuple, formatted once and reused for every packet
  std::vector<std::string> tup;
  if (format != EVR_WP_UNFORMATTED_V1) {
    tup.resize((size_t)N);
    char b[24];
    for (int64_t row = 0; row < N; ++row) {
      const int64_t k = row % P.Np;
      std::string& t = tup[(size_t)row];
      for (int i = 0; i < D; ++i) {
        snprintf(b, sizeof b, " %d", P.packed[(size_t)k * D + i]);
        t += b;
      }
      snprintf(b, sizeof b, " %d %d", 1, (int)(row / P.Np) + 1);
      t += b;
    }
  }
  auto tuple = [&](int64_t row, std::string& t) { t += tup[(size_t)row]; };
  bool ok = true;
  if (format == EVR_WP_UNFORMATTED_V1) {
    const char X = 'X';
    const int32_t hdr[3] = {npsi, (int32_t)N, 1};
    ok = put_record(o.f, &X, 1) && put_record(o.f, &hdr[0], 4) && put_record(o.f, &hdr[1], 4) &&
         put_record(o.f, &hdr[2], 4) && put_record(o.f, &X, 1);
    std::vector<int32_t> nd(D + 2);
    for (int64_t row = 0; row < N && ok; ++row) {
      const int64_t k = row % P.Np;
      for (int i = 0; i < D; ++i) nd[i] = P.packed[(size_t)k * D + i];
      nd[D] = 1;
      nd[D + 1] = (int32_t)(row / P.Np) + 1;
      ok = put_record(o.f, nd.data(), sizeof(int32_t) * (D + 2));
    }
    std::vector<double> v((size_t)N * (cplx ? 2 : 1));
    for (int j = 0; j < npsi && ok; ++j) {
      std::copy(psi + (cplx ? 2 : 1) * ld * j, psi + (cplx ? 2 : 1) * ld * j + v.size(), v.begin());
      ok = put_record(o.f, v.data(), v.size() * sizeof(double));
    }
  } else if (format == EVR_WP_FORMATTED_V1) {
    char b[160];
    snprintf(b, sizeof b, "&HEADERFILE\n VERSION_FILE=1,\n NB_PSI=%d,\n NB_TOT=%lld,\n /\n", npsi, (long long)N);
    s += b;
    for (int64_t row = 0; row < N && ok; ++row) {
      tuple(row, s);
      s += '\n';
      if (s.size() > (1 << 20)) ok = flush();
    }
    for (int j = 0; j < npsi && ok; ++j) {
      for (int64_t k = 0; k < N; ++k) {
        if (cplx) {
          s += " (";
          put_real(s, val(psi, ld, 1, j, k, 0));
          s += ",";
          put_real(s, val(psi, ld, 1, j, k, 1));
          s += ")";
        } else {
          put_real(s, val(psi, ld, 0, j, k, 0));
        }
        if ((k + 1) % (cplx ? 2 : 4) == 0 || k + 1 == N) s += '\n';
        if (s.size() > (1 << 20) && !(ok = flush())) break;
      }
    }
  } else {  // version 0 (all entries) or sparse (entries of modulus >= epsi), "end wp" lines
    char b[64];
    if (format == EVR_WP_FORMATTED_V0) snprintf(b, sizeof b, " %d %lld\n", npsi, (long long)N);
    else snprintf(b, sizeof b, " %d\n", npsi);
    s += b;
    for (int j = 0; j < npsi && ok; ++j) {
      for (int64_t row = 0; row < N; ++row) {
        const double a = val(psi, ld, cplx, j, row, 0), im = cplx ? val(psi, ld, cplx, j, row, 1) : 0.0;
        const double mod = cplx ? std::sqrt(a * a + im * im) : std::fabs(a);
        if (format == EVR_WP_SPARSE && !(mod >= epsi)) continue;
        tuple(row, s);
        put_real(s, a);
        if (cplx) put_real(s, im);
        s += '\n';
        if (s.size() > (1 << 20) && !(ok = flush())) break;
      }
      snprintf(b, sizeof b, " end wp %d\n", j + 1);
      s += b;
    }
  }
  ok = ok && flush();
  if (!ok || ferror(o.f)) return set_error(c, EVR_EINVAL, std::string("evr_psi_write: write error on ") + path);
  if (fclose(o.f) != 0) {
    o.f = nullptr;
    return set_error(c, EVR_EINVAL, std::string("evr_psi_write: close error on ") + path);
  }
  o.f = nullptr;
  return EVR_OK;
}

extern "C" int evr_psi_read(evr_ctx* c, const char* path, double* psi, int64_t ld, int npsi_max, int cplx,
                            int* npsi_read, int64_t* n_dropped) {
  if (int rc = check_ctx(c, "evr_psi_read")) return rc;
  const HostProblem& P = c->hp;
  if (!path || !psi || npsi_max < 0 || ld < P.Np * P.nb0 || (cplx != 0 && cplx != 1))
    return set_error(c, EVR_EINVAL, "evr_psi_read: null pointer, ld < N, npsi_max < 0 or bad cplx");
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(c, EVR_EINVAL, std::string("evr_psi_read: cannot open ") + path);
  std::vector<unsigned char> buf;
  unsigned char chunk[1 << 16];
  size_t got;
  while ((got = fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
  const bool err = ferror(f) != 0;
  fclose(f);
  if (err) return set_error(c, EVR_EINVAL, std::string("evr_psi_read: read error on ") + path);
  Reader R(c, psi, ld, npsi_max, cplx);
  int rc;
  // an unformatted file starts with the record of the character 'X'
  const unsigned char xrec[5] = {1, 0, 0, 0, 'X'};
  if (buf.size() >= 5 && memcmp(buf.data(), xrec, 5) == 0) {
    rc = R.unformatted(buf);
  } else {
    std::vector<std::string> lines;
    size_t a = 0;
    for (size_t i = 0; i <= buf.size(); ++i)
      if (i == buf.size() || buf[i] == '\n') {
        size_t e = i;
        if (e > a && buf[e - 1] == '\r') --e;
        if (i < buf.size() || e > a) lines.emplace_back((const char*)buf.data() + a, e - a);
        a = i + 1;
      }
    rc = R.formatted(lines);
  }
  if (rc) return rc;
  if (npsi_read) *npsi_read = R.stored;
  if (n_dropped) *n_dropped = R.dropped;
  return EVR_OK;
}

// ---------------------------------------------------------------- restart and autocorrelation
namespace {

int read_text(const char* path, std::vector<std::string>& lines) {
  FILE* f = fopen(path, "rb");
  if (!f) return EVR_EINVAL;
  std::string all;
  char chunk[1 << 16];
  size_t got;
  while ((got = fread(chunk, 1, sizeof chunk, f)) > 0) all.append(chunk, got);
  const bool err = ferror(f) != 0;
  fclose(f);
  if (err) return EVR_EINVAL;
  size_t a = 0;
  for (size_t i = 0; i <= all.size(); ++i)
    if (i == all.size() || all[i] == '\n') {
      size_t e = i;
      if (e > a && all[e - 1] == '\r') --e;
      if (i < all.size() || e > a) lines.push_back(all.substr(a, e - a));
      a = i + 1;
    }
  return EVR_OK;
}

bool write_all(const char* path, const std::string& s, const char* mode) {
  FILE* f = fopen(path, mode);
  if (!f) return false;
  bool ok = s.empty() || fwrite(s.data(), 1, s.size(), f) == s.size();
  ok = (fclose(f) == 0) && ok;
  return ok;
}

}  // namespace

// SaveWP_restart (Source_ElVibRot/sub_propagation/sub_module_propagation.f90:376-424):
// "T nb_WP size" then each packet's CvecB as one list-directed record.
extern "C" int evr_restart_write(evr_ctx* c, const char* path, double t, const double* psi, int64_t ld, int npsi) {
  if (int rc = check_ctx(c, "evr_restart_write")) return rc;
  const int64_t N = c->hp.Np * c->hp.nb0;
  if (!path || !psi || npsi < 1 || ld < N) return set_error(c, EVR_EINVAL, "evr_restart_write: bad arguments");
  std::string s;
  char b[96];
  s.reserve((size_t)npsi * N * 56 + 64);
  put_real(s, t);
  snprintf(b, sizeof b, " %d %lld\n", npsi, (long long)N);
  s += b;
  for (int j = 0; j < npsi; ++j)
    for (int64_t k = 0; k < N; ++k) {
      s += " (";
      put_real(s, psi[2 * (k + ld * j)]);
      s += ",";
      put_real(s, psi[2 * (k + ld * j) + 1]);
      s += ")";
      if ((k + 1) % 2 == 0 || k + 1 == N) s += '\n';
    }
  if (!write_all(path, s, "w")) return set_error(c, EVR_EINVAL, std::string("evr_restart_write: cannot write ") + path);
  return EVR_OK;
}

// ReadWP_restart (:425-488): a file whose first record does not hold "T nb_WP size" means
// no restart (T = 0, packets untouched, *found = 0); a header whose nb_WP or size differ from
// npsi or N is an error (the reference STOPs).
extern "C" int evr_restart_read(evr_ctx* c, const char* path, double* t, double* psi, int64_t ld, int npsi,
                                int* found) {
  if (int rc = check_ctx(c, "evr_restart_read")) return rc;
  const int64_t N = c->hp.Np * c->hp.nb0;
  if (!path || !t || !psi || !found || npsi < 1 || ld < N) return set_error(c, EVR_EINVAL, "evr_restart_read: bad arguments");
  *found = 0;
  *t = 0.0;
  std::vector<std::string> lines;
  if (read_text(path, lines)) return set_error(c, EVR_EINVAL, std::string("evr_restart_read: cannot read ") + path);
  if (lines.empty()) return EVR_OK;
  std::vector<std::string> h = items_of(lines[0]);
  double t0;
  long long nw, sz;
  if (h.size() < 3 || !parse_real(h[0], &t0) || !parse_int(h[1], &nw) || !parse_int(h[2], &sz)) return EVR_OK;
  if (nw != npsi || sz != N)
    return set_error(c, EVR_EINVAL, "evr_restart_read: inconsistent sizes (file " + std::to_string(nw) + " x " +
                                        std::to_string(sz) + ", expected " + std::to_string(npsi) + " x " +
                                        std::to_string(N) + ")");
  std::vector<double> tmp((size_t)2 * N * npsi);
  int64_t e = 0;
  const int64_t total = N * npsi;
  for (size_t li = 1; li < lines.size() && e < total; ++li)
    for (const std::string& it : items_of(lines[li])) {
      long long rep;
      double re, im;
      if (!parse_value_item(it, 1, &rep, &re, &im))
        return set_error(c, EVR_EINVAL, "evr_restart_read: value '" + it + "' is not a complex (re,im) constant");
      for (long long r = 0; r < rep && e < total; ++r, ++e) {
        tmp[2 * e] = re;
        tmp[2 * e + 1] = im;
      }
      if (e >= total) break;
    }
  if (e < total) return set_error(c, EVR_EINVAL, "evr_restart_read: file ends before the last packet");
  for (int j = 0; j < npsi; ++j)
    for (int64_t k = 0; k < N; ++k) {
      psi[2 * (k + ld * j)] = tmp[2 * (j * N + k)];
      psi[2 * (k + ld * j) + 1] = tmp[2 * (j * N + k) + 1];
    }
  *t = t0;
  *found = 1;
  return EVR_OK;
}

// Write_AutoCorr / Read_AutoCorr (:548-578): one line "AutoCor T Re Im |C|" per time.
extern "C" int evr_autocorr_write(const char* path, const double* t, const double* cdot, int n, int append) {
  if (!path || n < 0 || (n > 0 && (!t || !cdot))) return EVR_EINVAL;
  std::string s;
  for (int i = 0; i < n; ++i) {
    s += " AutoCor ";
    put_real(s, t[i]);
    put_real(s, cdot[2 * i]);
    put_real(s, cdot[2 * i + 1]);
    put_real(s, std::hypot(cdot[2 * i], cdot[2 * i + 1]));
    s += '\n';
  }
  return write_all(path, s, append ? "a" : "w") ? EVR_OK : EVR_EINVAL;
}

// Lines that do not read as "name T Re Im |C|" are skipped (Read_AutoCorr gives them 0).
extern "C" int evr_autocorr_read(const char* path, double* t, double* cdot, int n_max, int* n) {
  if (!path || !n || n_max < 0 || (n_max > 0 && (!t || !cdot))) return EVR_EINVAL;
  std::vector<std::string> lines;
  if (read_text(path, lines)) return EVR_EINVAL;
  int k = 0;
  for (const std::string& L : lines) {
    if (k >= n_max) break;
    std::vector<std::string> it = items_of(L);
    double tt, a, b, m;
    if (it.size() < 5 || !parse_real(it[1], &tt) || !parse_real(it[2], &a) || !parse_real(it[3], &b) ||
        !parse_real(it[4], &m))
      continue;
    t[k] = tt;
    cdot[2 * k] = a;
    cdot[2 * k + 1] = b;
    ++k;
  }
  *n = k;
  return EVR_OK;
}
