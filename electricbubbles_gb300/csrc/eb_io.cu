// The reference's input deck and checkpoint files, host side:
//  * `bubbin`, read by READINI (electric.f:275-337): list-directed records
//      k / nd(1..k) / dt tfinal nplot / cap bondx bondy E0 / k x (ai bi thetax cx cy ncyc);
//    only the first deck of the file is read;
//  * the initial curves of GEOINIT and INITPARAM (electric.f:340-496) at equispaced theta;
//  * `geometry.data`, written by DUMPDATA and read by READDATA (electric.f:1360-1421):
//      list-directed  k nbk neq / nd(1..k)
//      '(e22.16,2x,e22.16)'  dt time / area0(k) / arcl0(k) / z(i) for every node.
// List-directed input is read as whitespace- or comma-separated tokens across lines, as
// Fortran does; list-directed integer output follows gfortran's 12-character fields.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "eb_internal.h"

namespace {

struct Tokens {
  std::vector<std::string> t;
  size_t i = 0;
  bool next(std::string& s) {
    if (i >= t.size()) return false;
    s = t[i++];
    return true;
  }
};

bool read_tokens(const char* path, Tokens& tk) {
  FILE* f = fopen(path, "r");
  if (!f) return false;
  std::string cur;
  int c;
  while ((c = fgetc(f)) != EOF) {
    if (std::isspace(c) || c == ',') {
      if (!cur.empty()) tk.t.push_back(cur), cur.clear();
    } else {
      cur.push_back((char)c);
    }
  }
  if (!cur.empty()) tk.t.push_back(cur);
  fclose(f);
  return true;
}

// Fortran real: also accepts the D exponent letter and an exponent written without a
// letter (the Ew.d form of exponents beyond 99, e.g. 0.3000000000000000+121)
bool to_double(const std::string& s, double& v) {
  std::string u = s;
  bool has_e = false;
  for (char& ch : u) {
    if (ch == 'd' || ch == 'D') ch = 'e';
    if (ch == 'e' || ch == 'E') has_e = true;
  }
  if (!has_e) {
    size_t pos = u.find_last_of("+-");
    if (pos != std::string::npos && pos > 0 && (std::isdigit((unsigned char)u[pos - 1]) || u[pos - 1] == '.'))
      u.insert(pos, 1, 'e');
  }
  char* end = nullptr;
  errno = 0;
  v = strtod(u.c_str(), &end);
  return end && *end == '\0' && errno == 0;
}

bool to_int(const std::string& s, int& v) {
  char* end = nullptr;
  errno = 0;
  long x = strtol(s.c_str(), &end, 10);
  if (!end || *end != '\0' || errno != 0) return false;
  v = (int)x;
  return true;
}

// Fortran Ew.d output (w = 22, d = 16): 0.ddddddddddddddddE+xx, the optional leading
// zero dropped when the sign needs its column.
std::string fmt_e22_16(double x) {
  char buf[64];
  if (x == 0.0) return std::string("0.0000000000000000E+00");
  snprintf(buf, sizeof(buf), "%.15e", std::fabs(x));  // d.ddddddddddddddde+XX
  std::string m(buf);
  size_t epos = m.find('e');
  std::string digits = m.substr(0, 1) + m.substr(2, epos - 2);  // 16 significant digits
  int ex = atoi(m.c_str() + epos + 1) + 1;
  char eb[16];
  if (std::abs(ex) <= 99) snprintf(eb, sizeof(eb), "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
  else snprintf(eb, sizeof(eb), "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
  std::string body = "." + digits + eb;
  return x < 0 ? "-" + body : "0" + body;
}

// INITPARAM (electric.f:441-496): point and first two theta-derivatives of drop curve
void initparam(double th, double ai, double bi, double thetax, int ncyc, double& xp, double& yp,
               double& xd, double& yd, double& xdd, double& ydd) {
  if (ncyc == 0) {
    double cs = std::cos(th - thetax), sn = std::sin(th - thetax);
    double a2 = ai * ai, b2 = bi * bi;
    double rn = std::sqrt(b2 * cs * cs + a2 * sn * sn);
    double radius = ai * bi / rn;
    double rdot = -ai * bi * cs * sn * (a2 - b2) / (rn * rn * rn);
    double rddot = -ai * bi *
                   (2.0 * a2 * b2 * cs * cs * sn * sn + a2 * a2 * std::pow(cs, 4) + a2 * b2 - a2 * a2 +
                    b2 * b2 * std::pow(cs, 4) - 2.0 * b2 * b2 * cs * cs) /
                   std::pow(rn, 5);
    double c = std::cos(th), s = std::sin(th);
    xp = radius * c;
    yp = radius * s;
    xd = rdot * c - radius * s;
    yd = rdot * s + radius * c;
    xdd = rddot * c - 2.0 * rdot * s - radius * c;
    ydd = rddot * s + 2.0 * rdot * c - radius * s;
  } else if (ncyc < 0) {
    const double R = ai, nu = bi, q = std::sqrt(1.0 + nu * nu), r2 = std::sqrt(2.0);
    double den = (1.0 - 2.0 * nu * std::cos(2.0 * th) + nu * nu) * q;
    double ddot = 4.0 * nu * std::sin(2.0 * th) * q;
    double dddot = 8.0 * nu * std::cos(2.0 * th) * q;
    double fx = (1.0 - nu * nu) * (1.0 - nu) * R * r2, fy = (1.0 - nu * nu) * (1.0 + nu) * R * r2;
    xp = fx * std::cos(th) / den;
    yp = fy * std::sin(th) / den;
    xd = -fx * std::sin(th) / den - xp * ddot / den;
    xdd = -xp + fx * std::sin(th) * ddot / (den * den) - xd * ddot / den - xp * dddot / den +
          xp * ddot * ddot / (den * den);
    yd = fy * std::cos(th) / den - yp * ddot / den;
    ydd = -yp - fy * std::cos(th) * ddot / (den * den) - yd * ddot / den - yp * dddot / den +
          yp * ddot * ddot / (den * den);
  } else {
    double cs = std::cos(th), sn = std::sin(th), snn = std::sin(ncyc * th), csn = std::cos(ncyc * th);
    xp = ai * cs + bi * csn;
    yp = ai * sn - bi * snn;
    xd = -ai * sn - ncyc * bi * snn;
    xdd = -ai * cs - (double)ncyc * ncyc * bi * csn;
    yd = ai * cs - ncyc * bi * csn;
    ydd = -ai * sn + (double)ncyc * ncyc * bi * snn;
  }
}

}  // namespace

int eb_bubbin_read(const char* path, int kmax, int* k, int* nd, double* params, double* drops) {
  if (!path || !k || !nd || !params || !drops || kmax <= 0) return EB_ERR_ARG;
  Tokens tk;
  if (!read_tokens(path, tk)) {
    eb_set_last_error_msg("cannot open the input deck");
    return EB_ERR_ARG;
  }
  std::string s;
  auto bad = [](const char* what) {
    eb_set_last_error_msg(what);
    return EB_ERR_ARG;
  };
  int kk = 0;
  if (!tk.next(s) || !to_int(s, kk) || kk <= 0) return bad("deck: bad drop count k");
  if (kk > kmax) return bad("deck: more drops than kmax");
  for (int b = 0; b < kk; ++b)
    if (!tk.next(s) || !to_int(s, nd[b]) || nd[b] <= 0) return bad("deck: bad nd");
  double v[7];
  for (int i = 0; i < 7; ++i)
    if (!tk.next(s) || !to_double(s, v[i])) return bad("deck: bad dt/tfinal/nplot/cap/bond/E0 record");
  for (int i = 0; i < 7; ++i) params[i] = v[i];
  for (int b = 0; b < kk; ++b) {
    for (int i = 0; i < 5; ++i)
      if (!tk.next(s) || !to_double(s, drops[6 * b + i])) return bad("deck: bad drop record");
    int nc = 0;
    if (!tk.next(s) || !to_int(s, nc)) return bad("deck: bad ncyc");
    drops[6 * b + 5] = (double)nc;
  }
  *k = kk;
  return EB_OK;
}

int eb_geoinit(int k, const int* nd, const double* drops, double* z, double* dsdth, double* kappa,
               double* area0) {
  if (k <= 0 || !nd || !drops || !z) return EB_ERR_ARG;
  size_t ist = 0;
  for (int b = 0; b < k; ++b) {
    const double* d = drops + 6 * b;
    const double ai = d[0], bi = d[1], thetax = d[2], cx = d[3], cy = d[4];
    const int ncyc = (int)std::lround(d[5]);
    const double dth = 2.0 * EB_PI / nd[b];
    if (area0) area0[b] = ncyc == 0 ? EB_PI * ai * bi : EB_PI * (ai * ai - ncyc * bi * bi);
    for (int i = 0; i < nd[b]; ++i) {
      double xp, yp, xd, yd, xdd, ydd;
      initparam(dth * i, ai, bi, thetax, ncyc, xp, yp, xd, yd, xdd, ydd);
      z[2 * (ist + i)] = cx + xp;
      z[2 * (ist + i) + 1] = cy + yp;
      double sd = std::sqrt(xd * xd + yd * yd);
      if (dsdth) dsdth[ist + i] = sd;
      if (kappa) kappa[ist + i] = (xd * ydd - yd * xdd) / (sd * sd * sd);
    }
    ist += nd[b];
  }
  return EB_OK;
}

int eb_dumpdata(const char* path, int k, const int* nd, double dt, double time, const double* area0,
                const double* arcl0, const double* z) {
  if (!path || k <= 0 || !nd || !area0 || !arcl0 || !z) return EB_ERR_ARG;
  FILE* f = fopen(path, "w");
  if (!f) {
    eb_set_last_error_msg("cannot open the dump file");
    return EB_ERR_ARG;
  }
  long nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  fprintf(f, "%12d%12ld%12ld\n", k, nbk, 2 * nbk);
  for (int b = 0; b < k; ++b) fprintf(f, "%12d", nd[b]);
  fprintf(f, "\n");
  fprintf(f, "%s  %s\n", fmt_e22_16(dt).c_str(), fmt_e22_16(time).c_str());
  for (int b = 0; b < k; ++b) fprintf(f, "%s\n", fmt_e22_16(area0[b]).c_str());
  for (int b = 0; b < k; ++b) fprintf(f, "%s\n", fmt_e22_16(arcl0[b]).c_str());
  for (long i = 0; i < nbk; ++i) fprintf(f, "%s  %s\n", fmt_e22_16(z[2 * i]).c_str(), fmt_e22_16(z[2 * i + 1]).c_str());
  int bad = ferror(f);
  if (fclose(f) != 0 || bad) {
    eb_set_last_error_msg("write of the dump file failed");
    return EB_ERR_ARG;
  }
  return EB_OK;
}

int eb_readdata(const char* path, int kmax, long nmax, int* k, int* nd, double* dt, double* time,
                double* area0, double* arcl0, double* z) {
  if (!path || !k || !nd || !dt || !time || !area0 || !arcl0 || !z || kmax <= 0) return EB_ERR_ARG;
  Tokens tk;
  if (!read_tokens(path, tk)) {
    eb_set_last_error_msg("cannot open the dump file");
    return EB_ERR_ARG;
  }
  std::string s;
  auto bad = [](const char* what) {
    eb_set_last_error_msg(what);
    return EB_ERR_ARG;
  };
  int kk = 0, nbk = 0, neq = 0;
  if (!tk.next(s) || !to_int(s, kk) || kk <= 0 || kk > kmax) return bad("dump: bad k");
  if (!tk.next(s) || !to_int(s, nbk) || !tk.next(s) || !to_int(s, neq)) return bad("dump: bad nbk/neq");
  long tot = 0;
  for (int b = 0; b < kk; ++b) {
    if (!tk.next(s) || !to_int(s, nd[b]) || nd[b] <= 0) return bad("dump: bad nd");
    tot += nd[b];
  }
  if (tot != nbk || neq != 2 * nbk) return bad("dump: nd, nbk and neq disagree");
  if (tot > nmax) return bad("dump: more nodes than nmax");
  if (!tk.next(s) || !to_double(s, *dt) || !tk.next(s) || !to_double(s, *time)) return bad("dump: bad dt/time");
  for (int b = 0; b < kk; ++b)
    if (!tk.next(s) || !to_double(s, area0[b])) return bad("dump: bad area0");
  for (int b = 0; b < kk; ++b)
    if (!tk.next(s) || !to_double(s, arcl0[b])) return bad("dump: bad arcl0");
  for (long i = 0; i < 2 * tot; ++i)
    if (!tk.next(s) || !to_double(s, z[i])) return bad("dump: bad node coordinate");
  *k = kk;
  return EB_OK;
}
