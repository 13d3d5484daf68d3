// Host-side system setup: .mmp ingestion, topology, multipole rotation and the
// scaled-pair lists consumed by the GPU correction kernels.
//
// Reference behaviour restated here (file:line in the OpenMMPol sources):
//   .mmp reader            src/mod_inputloader.F90:15-257, 259-295
//   mmpol_prepare          src/mod_mmpol.F90:139-237
//   group adjacency        src/mod_mmpol.F90:272-323
//   thole_init             src/mod_electrostatics.F90:866-897
//   remove_null_pol        src/mod_electrostatics.F90:469-536
//   rotate_multipoles      src/rotate_multipoles.F90:232-464
//   screening rules        src/mod_electrostatics.F90:3338-3487
// The connectivity layers C_1..C_4 are built here by breadth-first search,
// which yields the same exact-distance sets as the reference's boolean
// sparse-matrix recursion C_n = C_{n-1} C_1 - (C_{n-1} + C_{n-2})
// (src/mod_adjacency_mat.F90:367-422).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <thread>

#include "ommp_internal.h"

namespace ommp {

namespace {

// Fortran list-directed input over a text file held in memory: a read of K
// values consumes records until K values are found and drops the rest of the
// last record.  Supports blank/comma separators, 'D' exponents and r*c
// repeat counts.  Numbers of at most 2^53 significant units with a decimal
// exponent within +-22 take Clinger's exact fast path (one correctly rounded
// multiplication or division by an exact power of ten, the same double as
// strtod); everything else goes through strtod.
class ListReader {
  static constexpr int kMaxLine = 128;  // values per read of the row readers

 public:
  explicit ListReader(std::vector<char> &&buf) : b_(std::move(buf)), p_(b_.data()), e_(b_.data() + b_.size()) {}
  bool skip(long n) {
    for (long i = 0; i < n; ++i)
      if (!next_line()) return false;
    return true;
  }
  bool values(double *out, int want) {
    int got = 0;
    while (got < want) {
      if (!next_line()) return false;
      const int k = line_values(ls_, le_, out + got, want - got);
      if (k < 0) return false;
      got += k;
    }
    return true;
  }
  // `rows` reads of `want` values each (row r into out[r * want ...]).  When
  // every one of the next `rows` records holds at least `want` values, each
  // read is exactly one record and the records are parsed on several
  // threads; otherwise the reads run one after the other.
  bool values_rows(double *out, int want, int rows) { return rows_parallel(out, want, rows); }
  bool ints_rows(int *out, int want, int rows) { return rows_parallel(out, want, rows); }
  // integers: plain digit tokens are converted directly; a record holding
  // anything else is read through values()
  bool ints(int *out, int want) {
    const char *save_p = p_;
    int got = 0;
    while (got < want) {
      if (!next_line()) return false;
      const char *p = ls_;
      bool plain = true;
      while (p < le_ && got < want) {
        while (p < le_ && sep(*p)) ++p;
        if (p >= le_) break;
        bool neg = false;
        if (*p == '-' || *p == '+') neg = *p++ == '-';
        const char *d0 = p;
        long v = 0;
        while (p < le_ && *p >= '0' && *p <= '9' && p - d0 < 9) v = v * 10 + (*p++ - '0');
        if (p == d0 || (p < le_ && !sep(*p))) {
          plain = false;
          break;
        }
        out[got++] = (int)(neg ? -v : v);
      }
      if (!plain) {  // repeat counts, decimals, exponents: the general reader
        p_ = save_p;
        buf_.resize(want);
        if (!values(buf_.data(), want)) return false;
        for (int i = 0; i < want; ++i) out[i] = (int)buf_[i];
        return true;
      }
    }
    return true;
  }

 private:
  bool next_line() {
    if (p_ >= e_) return false;
    ls_ = p_;
    const char *nl = static_cast<const char *>(memchr(p_, '\n', e_ - p_));
    le_ = nl ? nl : e_;
    p_ = nl ? nl + 1 : e_;
    return true;
  }
  static bool sep(char c) { return c == ' ' || c == ',' || (c >= '\t' && c <= '\r'); }
  // up to `want` values of the record [p, e); the count, or -1 on a bad token
  static int line_values(const char *p, const char *e, double *out, int want) {
    int got = 0;
    while (p < e && got < want) {
      while (p < e && sep(*p)) ++p;
      if (p >= e) break;
      const char *t = p;
      while (p < e && !sep(*p)) ++p;
      long rep = 1;
      const char *num = t;
      for (const char *q = t; q < p; ++q)
        if (*q == '*') {
          rep = 0;
          for (const char *d = t; d < q; ++d) {
            if (*d < '0' || *d > '9') return -1;
            rep = rep * 10 + (*d - '0');
          }
          if (rep <= 0) return -1;
          num = q + 1;
          break;
        }
      double v;
      if (!number(num, p, v)) return -1;
      for (long r = 0; r < rep && got < want; ++r) out[got++] = v;
    }
    return got;
  }
  static int line_values(const char *p, const char *e, int *out, int want) {
    int got = 0;
    while (p < e && got < want) {
      while (p < e && sep(*p)) ++p;
      if (p >= e) break;
      bool neg = false;
      const char *t = p;
      if (*p == '-' || *p == '+') neg = *p++ == '-';
      const char *d0 = p;
      long v = 0;
      while (p < e && *p >= '0' && *p <= '9' && p - d0 < 9) v = v * 10 + (*p++ - '0');
      if (p == d0 || (p < e && !sep(*p))) {  // not a plain integer: general parse of the rest
        double tmp[kMaxLine];
        const int k = line_values(t, e, tmp, std::min(want - got, kMaxLine));
        if (k < 0) return -1;
        for (int i = 0; i < k; ++i) out[got++] = (int)tmp[i];
        return got;
      }
      out[got++] = (int)(neg ? -v : v);
    }
    return got;
  }
  template <typename T>
  bool rows_parallel(T *out, int want, int rows) {
    const char *start = p_;
    std::vector<const char *> ls(rows), le(rows);
    bool enough = true;
    for (int r = 0; r < rows; ++r) {
      if (!next_line()) {
        enough = false;
        break;
      }
      ls[r] = ls_;
      le[r] = le_;
    }
    bool regular = enough && want <= kMaxLine;
    if (regular) {
      const int nt = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), rows / 2048));
      std::vector<char> ok(nt, 1);
      auto work = [&](int t) {
        const int r0 = (int)((long)rows * t / nt), r1 = (int)((long)rows * (t + 1) / nt);
        for (int r = r0; r < r1; ++r)
          if (line_values(ls[r], le[r], out + (size_t)r * want, want) != want) {
            ok[t] = 0;
            return;
          }
      };
      std::vector<std::thread> th;
      for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
      work(0);
      for (auto &x : th) x.join();
      for (char c : ok) regular = regular && c;
    }
    if (regular) return true;
    p_ = start;  // records shorter than a read: sequential list-directed reads
    for (int r = 0; r < rows; ++r)
      if (!read_one(out + (size_t)r * want, want)) return false;
    return true;
  }
  bool read_one(double *out, int want) { return values(out, want); }
  bool read_one(int *out, int want) { return ints(out, want); }
  static bool number(const char *s, const char *e, double &v) {
    static const double p10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                   1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    const char *q = s;
    bool neg = false;
    if (q < e && (*q == '+' || *q == '-')) neg = *q++ == '-';
    unsigned long long m = 0;
    int scale = 0;
    bool any = false, exact = true;
    for (; q < e && *q >= '0' && *q <= '9'; ++q, any = true)
      if (m < (1ull << 53) / 10) {
        m = m * 10 + (*q - '0');
      } else {
        exact = false;
      }
    if (q < e && *q == '.') {
      ++q;
      for (; q < e && *q >= '0' && *q <= '9'; ++q, any = true)
        if (m < (1ull << 53) / 10) {
          m = m * 10 + (*q - '0');
          --scale;
        } else {
          exact = false;
        }
    }
    if (any && q < e && (*q == 'e' || *q == 'E' || *q == 'd' || *q == 'D')) {
      ++q;
      bool eneg = false;
      if (q < e && (*q == '+' || *q == '-')) eneg = *q++ == '-';
      int x = 0;
      bool ed = false;
      for (; q < e && *q >= '0' && *q <= '9'; ++q, ed = true)
        if (x < 10000) x = x * 10 + (*q - '0');
      if (!ed) exact = false;
      scale += eneg ? -x : x;
    }
    if (any && exact && q == e && scale >= -22 && scale <= 22) {
      const double d = (double)m;
      v = scale < 0 ? d / p10[-scale] : d * p10[scale];
      if (neg) v = -v;
      return true;
    }
    // general path: strtod on a copy with Fortran 'D' exponents as 'e'
    char tok[128];
    const long n = std::min<long>(e - s, 127);
    for (long k = 0; k < n; ++k) tok[k] = (s[k] == 'D' || s[k] == 'd') ? 'e' : s[k];
    tok[n] = 0;
    char *end = nullptr;
    v = strtod(tok, &end);
    return end != tok;
  }
  std::vector<char> b_;
  const char *p_, *e_;
  const char *ls_ = nullptr, *le_ = nullptr;
  std::vector<double> buf_;
};

constexpr int kMaxN12 = 8;    // mod_inputloader.F90:65
constexpr int kMaxPgp = 120;  // mod_inputloader.F90:67

// Exact bond-distance layers 1..depth from every row of `adj` (BFS).  Rows
// are independent: ranges of rows run on several threads and their pieces
// are joined in row order.
void distance_layers(const Csr &adj, int depth, Csr *layers) {
  const int n = adj.n;
  const int nt = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), n / 4096));
  struct Piece {
    std::vector<int> ci[4];
    std::vector<int> len[4];
  };
  std::vector<Piece> pieces(nt);
  auto work = [&](int t) {
    const int r0 = (int)((long)n * t / nt), r1 = (int)((long)n * (t + 1) / nt);
    Piece &pc = pieces[t];
    std::vector<int> dist(n, -1), touched;
    std::vector<std::vector<int>> rows(depth);
    std::deque<int> q;
    for (int s = r0; s < r1; ++s) {
      for (auto &r : rows) r.clear();
      q.assign(1, s);
      dist[s] = 0;
      touched.assign(1, s);
      while (!q.empty()) {
        int a = q.front();
        q.pop_front();
        if (dist[a] == depth) continue;
        for (int k = adj.ri[a]; k < adj.ri[a + 1]; ++k) {
          int b = adj.ci[k];
          if (dist[b] >= 0) continue;
          dist[b] = dist[a] + 1;
          touched.push_back(b);
          rows[dist[b] - 1].push_back(b);
          q.push_back(b);
        }
      }
      for (int l = 0; l < depth; ++l) {
        std::sort(rows[l].begin(), rows[l].end());
        pc.ci[l].insert(pc.ci[l].end(), rows[l].begin(), rows[l].end());
        pc.len[l].push_back((int)rows[l].size());
      }
      for (int x : touched) dist[x] = -1;
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
  work(0);
  for (auto &x : th) x.join();
  for (int l = 0; l < depth; ++l) {
    layers[l].n = n;
    layers[l].ri.assign(n + 1, 0);
    layers[l].ci.clear();
    int row = 0;
    for (auto &pc : pieces) {
      layers[l].ci.insert(layers[l].ci.end(), pc.ci[l].begin(), pc.ci[l].end());
      for (int len : pc.len[l]) {
        layers[l].ri[row + 1] = layers[l].ri[row] + len;
        ++row;
      }
    }
  }
}

// Position of `j` in the distance layers of row `i`: 1..4, or 0 if farther.
int layer_of(const Csr *layers, int nlev, int i, int j) {
  for (int l = 0; l < nlev; ++l)
    if (layers[l].has(i, j)) return l + 1;
  return 0;
}

}  // namespace

bool read_mmp(const std::string &path, HostModel &m, std::string &err) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) {
    err = "Input file '" + path + "' does not exist.";
    return false;
  }
  std::vector<char> text;
  {
    long size = -1;
    if (fseek(f, 0, SEEK_END) == 0) size = ftell(f);
    if (size >= 0 && fseek(f, 0, SEEK_SET) == 0) {
      text.resize((size_t)size);
      text.resize(fread(text.data(), 1, text.size(), f));
    } else {  // not seekable: read in chunks
      char chunk[1 << 16];
      size_t got;
      while ((got = fread(chunk, 1, sizeof chunk, f)) > 0) text.insert(text.end(), chunk, chunk + got);
    }
    fclose(f);
  }
  ListReader r(std::move(text));
  auto fail = [&](const char *what) {
    err = std::string("error while reading MMP file '") + path + "': " + what;
    return false;
  };
  double v[4];
  if (!r.values(v, 1)) return fail("revision");
  int rev = (int)v[0];
  if (rev != 2 && rev != 3) {
    err = "MMP file is only supported with version 2 or 3.";
    return false;
  }
  if (!r.skip(2) || !r.values(v, 1)) return fail("ff_type");
  int ff_type = (int)v[0];
  if (!r.values(v, 1)) return fail("ff_rules");
  int ff_rules = (int)v[0];
  if (!r.skip(rev == 3 ? 17 : 15) || !r.values(v, 1)) return fail("mm_atoms");
  int mm = (int)v[0];
  if (mm <= 0) return fail("mm_atoms");
  m = HostModel();
  m.amoeba = (ff_type == 1);
  m.mm = mm;
  m.ld_cart = m.amoeba ? 10 : 1;
  m.n_ipd = m.amoeba ? 2 : 1;
  m.fmm_requested = mm > 1000;
  m.cmm.resize(3 * (size_t)mm);
  m.q.resize((size_t)m.ld_cart * mm);
  std::vector<double> pol(mm);
  if (!r.skip(mm + 1)) return fail("atomic numbers");
  if (!r.values_rows(m.cmm.data(), 3, mm)) return fail("coordinates");
  if (!r.skip(mm)) return fail("residues");
  if (!r.values_rows(m.q.data(), m.ld_cart, mm)) return fail("multipoles");
  if (!r.values_rows(pol.data(), 1, mm)) return fail("polarizabilities");
  for (auto &c : m.cmm) c *= kAng2Au;
  for (int i = 0; i < mm; ++i)
    if (pol[i] > 1e-8) {
      m.polar_mm.push_back(i);
      m.pol.push_back(m.amoeba ? pol[i] * kAng2Au * kAng2Au * kAng2Au : pol[i]);
    }
  m.npol = (int)m.pol.size();
  // scale factors (mod_constants.F90:37-52; mod_inputloader.F90:175-200)
  if (m.amoeba) {
    const double ms[4] = {0, 0, 0.4, 0.8}, ps[4] = {0, 0, 1, 1}, ds[4] = {0, 1, 1, 1},
                 us[4] = {1, 1, 1, 1}, pi[4] = {0, 0, 0.5, 1};
    memcpy(m.mscale, ms, sizeof ms);
    memcpy(m.pscale, ps, sizeof ps);
    memcpy(m.dscale, ds, sizeof ds);
    memcpy(m.uscale, us, sizeof us);
    memcpy(m.pscale_intra, pi, sizeof pi);
    m.thole_scale = 0.0;
  } else {
    const double al[4] = {0, 0, 1, 1}, dl[4] = {1, 1, 1, 1};
    const double *s = (ff_rules == 1) ? dl : al;
    memcpy(m.mscale, s, 4 * sizeof(double));
    memcpy(m.pscale, s, 4 * sizeof(double));
    memcpy(m.dscale, s, 4 * sizeof(double));
    memcpy(m.uscale, s, 4 * sizeof(double));
    m.thole_scale = (ff_rules == 1) ? 2.0580 : 2.5874;
  }
  // 1-2 connectivity, 8 entries per atom, 0 = none
  Csr &adj = m.conn[0];
  adj.n = mm;
  adj.ri.assign(mm + 1, 0);
  adj.ci.clear();
  std::vector<int> conn12((size_t)kMaxN12 * mm);
  if (!r.ints_rows(conn12.data(), kMaxN12, mm)) return fail("connectivity");
  for (int i = 0; i < mm; ++i) {
    const int *row = &conn12[(size_t)kMaxN12 * i];
    std::vector<int> nb;
    for (int k = 0; k < kMaxN12; ++k)
      if (row[k] != 0) {
        if (row[k] < 1 || row[k] > mm) return fail("connectivity index out of range");
        nb.push_back(row[k] - 1);
      }
    std::sort(nb.begin(), nb.end());
    adj.ci.insert(adj.ci.end(), nb.begin(), nb.end());
    adj.ri[i + 1] = (int)adj.ci.size();
  }
  m.grp.assign(mm, 0);
  m.frame.assign(mm, 0);
  m.iz.assign(mm, -1);
  m.ix.assign(mm, -1);
  m.iy.assign(mm, -1);
  if (m.amoeba) {
    // polarization groups: first listing assigns the group id (polgroup11_to_mm2pg)
    std::vector<int> lists((size_t)kMaxPgp * mm);
    if (!r.ints_rows(lists.data(), kMaxPgp, mm)) return fail("polarization groups");
    std::fill(m.grp.begin(), m.grp.end(), -1);
    int g = 0;
    for (int i = 0; i < mm; ++i) {
      if (m.grp[i] != -1) continue;
      for (int k = 0; k < kMaxPgp; ++k) {
        int a = lists[(size_t)kMaxPgp * i + k];
        if (a == 0) break;
        if (a < 1 || a > mm || m.grp[a - 1] != -1) return fail("inconsistent polarization groups");
        m.grp[a - 1] = g;
      }
      ++g;
    }
    for (int i = 0; i < mm; ++i)
      if (m.grp[i] < 0) return fail("atom without polarization group");
    m.ngrp = g;
    std::vector<int> frames(4 * (size_t)mm);
    if (!r.ints_rows(frames.data(), 4, mm)) return fail("multipole frames");
    for (int i = 0; i < mm; ++i) {
      const int *t = &frames[4 * (size_t)i];
      m.frame[i] = t[0];
      m.iz[i] = t[1] - 1;
      m.ix[i] = t[2] - 1;
      m.iy[i] = t[3] - 1;
      for (int k = 1; k < 4; ++k)
        if (t[k] < 0 || t[k] > mm) return fail("frame atom index out of range");
    }
    m.damping.assign(m.npol, 0.39);  // .mmp input forces a = 0.39 (:247)
  } else {
    m.damping.assign(m.npol, 0.0);
  }
  return true;
}

bool rotate_multipoles(HostModel &m, std::string &err) {
  // Lab-frame multipoles q from the local-frame set q0; frame axes from the
  // z/x/y reference atoms: ez along u, ex from v by Gram-Schmidt, ey = ez x ex.
  for (int j = 0; j < m.mm; ++j) {
    auto C = [&](int a) { return &m.cmm[3 * (size_t)a]; };
    const double *c = C(j);
    const double *cz = C(m.iz[j] >= 0 ? m.iz[j] : j);
    const double *cx = C(m.ix[j] >= 0 ? m.ix[j] : j);
    const double *cy = C(m.iy[j] >= 0 ? m.iy[j] : j);
    double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    int fr = m.frame[j];
    if (fr != 0) {
      double a[3], b[3], d[3];
      for (int k = 0; k < 3; ++k) {
        a[k] = cz[k] - c[k];
        b[k] = cx[k] - c[k];
        d[k] = cy[k] - c[k];
      }
      auto nrm = [](const double *x) { return std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]); };
      double na = nrm(a), nb = nrm(b), nd = nrm(d);
      double u[3] = {0, 0, 0}, v[3] = {0, 0, 0};
      switch (fr) {
        case 1:  // z-then-x
          for (int k = 0; k < 3; ++k) u[k] = a[k], v[k] = b[k];
          break;
        case 2:  // bisector
          for (int k = 0; k < 3; ++k) u[k] = nb * a[k] + na * b[k], v[k] = b[k];
          break;
        case 3:  // z-only
          for (int k = 0; k < 3; ++k) u[k] = a[k];
          if (u[2] / na <= 0.866 && std::fabs(u[1]) > kEpsRp)
            v[0] = 1.0;
          else
            v[1] = 1.0;
          break;
        case 4:  // z-bisector
          for (int k = 0; k < 3; ++k) u[k] = a[k], v[k] = nd * b[k] + nb * d[k];
          break;
        case 5:  // 3-fold
          for (int k = 0; k < 3; ++k) u[k] = nb * nd * a[k] + na * nd * b[k] + na * nb * d[k], v[k] = b[k];
          break;
        default:
          break;
      }
      double nu = nrm(u), nv = nrm(v);
      if (nu < kEpsRp || nv < kEpsRp) {
        err = "Ill defined rotation axis (either u or v vectors have 0 norm.";
        return false;
      }
      double ez[3], ex[3], ey[3];
      for (int k = 0; k < 3; ++k) ez[k] = u[k] / nu;
      double vez = v[0] * ez[0] + v[1] * ez[1] + v[2] * ez[2];
      for (int k = 0; k < 3; ++k) ex[k] = v[k] - vez * ez[k];
      double nx = nrm(ex);
      for (int k = 0; k < 3; ++k) ex[k] /= nx;
      ey[0] = ez[1] * ex[2] - ez[2] * ex[1];
      ey[1] = ez[2] * ex[0] - ez[0] * ex[2];
      ey[2] = ez[0] * ex[1] - ez[1] * ex[0];
      for (int k = 0; k < 3; ++k) R[k][0] = ex[k], R[k][1] = ey[k], R[k][2] = ez[k];
    }
    const double *s = &m.q0[10 * (size_t)j];
    double *t = &m.q[10 * (size_t)j];
    t[0] = s[0];
    for (int a = 0; a < 3; ++a) t[1 + a] = R[a][0] * s[1] + R[a][1] * s[2] + R[a][2] * s[3];
    // quadrupole xx,xy,yy,xz,yz,zz -> R Q R^T
    const double Q[3][3] = {{s[4], s[5], s[7]}, {s[5], s[6], s[8]}, {s[7], s[8], s[9]}};
    double RQ[3][3], O[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) RQ[a][b] = R[a][0] * Q[0][b] + R[a][1] * Q[1][b] + R[a][2] * Q[2][b];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) O[a][b] = RQ[a][0] * R[b][0] + RQ[a][1] * R[b][1] + RQ[a][2] * R[b][2];
    t[4] = O[0][0];
    t[5] = O[0][1];
    t[6] = O[1][1];
    t[7] = O[0][2];
    t[8] = O[1][2];
    t[9] = O[2][2];
  }
  return true;
}

bool prepare_model(HostModel &m, std::string &err) {
  {
    const Csr adj = m.conn[0];  // the layers overwrite conn[0]: read from a copy
    distance_layers(adj, 4, m.conn);
  }
  // remove_null_pol: |alpha| <= 100 eps is dropped
  {
    std::vector<double> pol;
    std::vector<int> pm;
    std::vector<double> damp;
    for (int k = 0; k < m.npol; ++k)
      if (std::fabs(m.pol[k]) > kEpsRp) {
        pol.push_back(m.pol[k]);
        pm.push_back(m.polar_mm[k]);
        damp.push_back(m.damping[k]);
      }
    m.pol.swap(pol);
    m.polar_mm.swap(pm);
    m.damping.swap(damp);
    m.npol = (int)m.pol.size();
  }
  m.mm_polar.assign(m.mm, -1);
  for (int k = 0; k < m.npol; ++k) m.mm_polar[m.polar_mm[k]] = k;
  // Thole factors: alpha^(1/6), times sqrt(thole_scale) for Wang
  m.thole.assign(m.mm, 0.0);
  for (int k = 0; k < m.npol; ++k) m.thole[m.polar_mm[k]] = std::pow(m.pol[k], 1.0 / 6.0);
  if (!m.amoeba) {
    if (!(m.thole_scale > kEpsRp)) {
      err = "Scale factor for Thole damping should be greater than 0.0 when non-AMOEBA FF are used";
      return false;
    }
    double sq = std::sqrt(m.thole_scale);
    for (auto &t : m.thole) t *= sq;
  }
  if (m.amoeba) {
    m.q0 = m.q;
    for (int i = 0; i < m.mm; ++i)
      for (int k = 4; k < 10; ++k) m.q0[10 * (size_t)i + k] /= 3.0;
    // group -> atoms
    Csr &ga = m.grp_atoms;
    ga.n = m.ngrp;
    ga.ri.assign(m.ngrp + 1, 0);
    for (int i = 0; i < m.mm; ++i) ga.ri[m.grp[i] + 1]++;
    for (int g = 0; g < m.ngrp; ++g) ga.ri[g + 1] += ga.ri[g];
    ga.ci.resize(m.mm);
    std::vector<int> fill(ga.ri.begin(), ga.ri.end() - 1);
    for (int i = 0; i < m.mm; ++i) ga.ci[fill[m.grp[i]]++] = i;
    // group adjacency through inter-group bonds, then layers 0..3
    Csr gadj;
    gadj.n = m.ngrp;
    gadj.ri.assign(m.ngrp + 1, 0);
    for (int g = 0; g < m.ngrp; ++g) {
      std::vector<int> nb;
      for (int k = ga.ri[g]; k < ga.ri[g + 1]; ++k) {
        int a = ga.ci[k];
        for (int l = m.conn[0].ri[a]; l < m.conn[0].ri[a + 1]; ++l) {
          int g2 = m.grp[m.conn[0].ci[l]];
          if (g2 != g && std::find(nb.begin(), nb.end(), g2) == nb.end()) nb.push_back(g2);
        }
      }
      std::sort(nb.begin(), nb.end());
      gadj.ci.insert(gadj.ci.end(), nb.begin(), nb.end());
      gadj.ri[g + 1] = (int)gadj.ci.size();
    }
    m.pg_conn[0].n = m.ngrp;
    m.pg_conn[0].ri.resize(m.ngrp + 1);
    m.pg_conn[0].ci.resize(m.ngrp);
    for (int g = 0; g <= m.ngrp; ++g) m.pg_conn[0].ri[g] = g;
    for (int g = 0; g < m.ngrp; ++g) m.pg_conn[0].ci[g] = g;
    distance_layers(gadj, 3, &m.pg_conn[1]);
    if (!rotate_multipoles(m, err)) return false;
  } else {
    m.q0 = m.q;
  }
  return true;
}

// Static->polarizable field scales for source mm atom i and target mm atom t.
// P field: connectivity rules (intra-group table for AMOEBA); D field
// (AMOEBA): polarization-group distance.  screening_rules :3420-3483.
void build_m2d_pairs(const HostModel &m, ScaledPairs &out) {
  out.ri.assign(m.npol + 1, 0);
  out.src.clear();
  out.sP.clear();
  out.sD.clear();
  std::vector<int> cand;
  for (int j = 0; j < m.npol; ++j) {
    int t = m.polar_mm[j];
    cand.clear();
    for (int l = 0; l < 4; ++l)
      for (int k = m.conn[l].ri[t]; k < m.conn[l].ri[t + 1]; ++k) cand.push_back(m.conn[l].ci[k]);
    if (m.amoeba) {
      int gt = m.grp[t];
      for (int l = 0; l < 4; ++l)
        for (int k = m.pg_conn[l].ri[gt]; k < m.pg_conn[l].ri[gt + 1]; ++k) {
          int g = m.pg_conn[l].ci[k];
          for (int a = m.grp_atoms.ri[g]; a < m.grp_atoms.ri[g + 1]; ++a) cand.push_back(m.grp_atoms.ci[a]);
        }
    }
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    for (int i : cand) {
      if (i == t) continue;  // the self pair never enters the field
      double sP = 1.0, sD = 1.0;
      int d = layer_of(m.conn, 4, t, i);
      if (d > 0) {
        if (m.amoeba && m.grp[i] == m.grp[t])
          sP = m.pscale_intra[d - 1];
        else
          sP = m.pscale[d - 1];
      }
      if (m.amoeba) {
        int gi = m.grp[i], gd = 0;
        for (int l = 0; l < 4; ++l)
          if (m.pg_conn[l].has(m.grp[t], gi)) {
            gd = l + 1;
            break;
          }
        if (gd > 0) sD = m.dscale[gd - 1];
      }
      bool keep = std::fabs(sP - 1.0) > kEpsRp || (m.amoeba && std::fabs(sD - 1.0) > kEpsRp);
      if (!keep) continue;
      // a scale that rounds to zero is skipped by the reference (todo flag)
      if (std::fabs(sP) <= kEpsRp) sP = 0.0;
      if (std::fabs(sD) <= kEpsRp) sD = 0.0;
      out.src.push_back(i);
      out.sP.push_back(sP);
      out.sD.push_back(m.amoeba ? sD : sP);
    }
    out.ri[j + 1] = (int)out.src.size();
  }
}

// Dipole-dipole scales (u-scale): candidates within four bonds; AMOEBA uses
// the polarization-group distance, other force fields the bond distance.
void build_d2d_pairs(const HostModel &m, ScaledPairs &out) {
  out.ri.assign(m.npol + 1, 0);
  out.src.clear();
  out.sP.clear();
  out.sD.clear();
  for (int j = 0; j < m.npol; ++j) {
    int t = m.polar_mm[j];
    for (int l = 0; l < 4; ++l)
      for (int k = m.conn[l].ri[t]; k < m.conn[l].ri[t + 1]; ++k) {
        int i = m.conn[l].ci[k];
        int ip = m.mm_polar[i];
        if (ip < 0) continue;
        double s = 1.0;
        if (m.amoeba) {
          for (int g = 0; g < 4; ++g)
            if (m.pg_conn[g].has(m.grp[t], m.grp[i])) {
              s = m.uscale[g];
              break;
            }
        } else {
          s = m.uscale[l];
        }
        if (std::fabs(s - 1.0) <= kEpsRp) continue;
        if (std::fabs(s) <= kEpsRp) s = 0.0;
        out.src.push_back(ip);
        out.sP.push_back(s);
        out.sD.push_back(s);
      }
    out.ri[j + 1] = (int)out.src.size();
  }
}

}  // namespace ommp
