// PIHM input decks (include/pihm_deck.h): the reference's text input files
// read and initialised on the host.
//
// Line rules follow the reference's reader utilities (src/custom_io.c:71-270):
// a line is skipped when it is empty or its first non-blank character is '#'
// or a line end, a UTF-8 byte-order mark at a line start is dropped, keywords
// compare case-insensitively, numbers are read as the reference's scanf
// formats read them.  The derivations restate InitTopo / InitSoil / InitLc /
// InitRiver / InitSurfL / CorrElev / RelaxIc with the same operations in the
// same order (the reference's pow(x, 2) is x * x; the C library's pow is
// called where the reference calls it), so a deck gives the reference's
// values bit for bit.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <memory>
#include <string>
#include <vector>

#include "pihm_deck.h"
#include "pihm_land.h"

namespace {

thread_local std::string g_error;

constexpr int kEdges = 3;
constexpr double kRivDpthMin = 0.05;  // RIVDPTHMIN, src/include/pihm_const.h:78
constexpr double kSatMin = 0.1;
constexpr double kCmcFactr = 2E-4;    // CMCFACTR, canopy water capacity per LAI (m), src/include/pihm_const.h:80
enum { kRectangle = 1, kTriangle = 2, kQuadratic = 3, kCubic = 4 };

struct DeckError {
  int code;
};

[[noreturn]] void fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_error = buf;
  throw DeckError{code};
}

// One text file read line by line with the reference's skipping rules.
class LineFile {
 public:
  explicit LineFile(const std::string &path) : path_(path) {
    f_ = std::fopen(path.c_str(), "r");
    if (!f_) fail(PIHM_DECK_ERR_IO, "cannot open %s", path.c_str());
  }
  ~LineFile() {
    if (f_) std::fclose(f_);
  }
  LineFile(const LineFile &) = delete;
  LineFile &operator=(const LineFile &) = delete;

  // The next readable line; false at the end of the file.
  bool next(std::string &line) {
    char buf[4096];
    while (std::fgets(buf, sizeof buf, f_)) {
      lno_++;
      char *p = buf;
      if ((unsigned char)p[0] == 0xEF && (unsigned char)p[1] == 0xBB && (unsigned char)p[2] == 0xBF) p += 3;
      if (readable(p)) {
        line = p;
        return true;
      }
    }
    return false;
  }
  std::string need(const char *what) {
    std::string line;
    if (!next(line)) fail(PIHM_DECK_ERR_FORMAT, "%s: unexpected end of file, expected %s", path_.c_str(), what);
    return line;
  }
  [[noreturn]] void bad(const char *what) {
    fail(PIHM_DECK_ERR_FORMAT, "%s near line %d: %s", path_.c_str(), lno_, what);
  }
  const std::string &path() const { return path_; }

 private:
  static bool readable(const char *s) {
    while (*s == ' ' || *s == '\t') s++;
    return *s && *s != '#' && *s != '\n' && *s != '\r';
  }
  std::string path_;
  FILE *f_ = nullptr;
  int lno_ = 0;
};

std::string first_token(const std::string &line) {
  char tok[1024] = {0};
  std::sscanf(line.c_str(), "%1023s", tok);
  return tok;
}

bool same_word(const std::string &a, const char *b) {
  if (a.size() != std::strlen(b)) return false;
  for (size_t k = 0; k < a.size(); k++)
    if (std::tolower((unsigned char)a[k]) != std::tolower((unsigned char)b[k])) return false;
  return true;
}

int keyword_int(LineFile &f, const char *key) {
  const std::string line = f.need(key);
  char tok[1024];
  int v;
  if (std::sscanf(line.c_str(), "%1023s %d", tok, &v) != 2 || !same_word(tok, key))
    f.bad((std::string("expected keyword ") + key).c_str());
  return v;
}

double keyword_double(LineFile &f, const char *key) {
  const std::string line = f.need(key);
  char tok[1024];
  double v;
  if (std::sscanf(line.c_str(), "%1023s %lf", tok, &v) != 2 || !same_word(tok, key))
    f.bad((std::string("expected keyword ") + key).c_str());
  return v;
}

// "YYYY-MM-DD hh:mm" (or a four-digit year) as seconds since 1970 UTC, as
// StrTime reads it (src/time_func.c:24-63)
int64_t parse_time(const char *ts1, const char *ts2, bool *ok) {
  std::tm tm{};
  const std::string s = std::string(ts1) + " " + ts2;
  int y, mo, d, h, mi;
  *ok = true;
  if (std::sscanf(s.c_str(), "%d-%d-%d %d:%d", &y, &mo, &d, &h, &mi) == 5 && s.size() == 16) {
    tm.tm_year = y - 1900;
    tm.tm_mon = mo - 1;
    tm.tm_mday = d;
    tm.tm_hour = h;
    tm.tm_min = mi;
  } else {
    *ok = false;
    return 0;
  }
  return (int64_t)timegm(&tm);
}

int64_t keyword_time(LineFile &f, const char *key) {
  const std::string line = f.need(key);
  char tok[1024], t1[256], t2[256];
  bool ok = false;
  int64_t t = 0;
  if (std::sscanf(line.c_str(), "%1023s %255s %255s", tok, t1, t2) == 3 && same_word(tok, key))
    t = parse_time(t1, t2, &ok);
  if (!ok) f.bad((std::string("expected keyword ") + key + " YYYY-MM-DD hh:mm").c_str());
  return t;
}

// A time series: knots and nvar values per knot (tsdata_struct).
struct Series {
  int nvar = 1;
  std::vector<int64_t> t;
  std::vector<double> v;  // [knot][nvar]
};

// Read the data lines of a series block until a line whose first token is
// one of the stop words, or the end of the file; returns that line (or "").
// A data line is a time stamp and nvar numbers (ReadTS, src/read_func.c:3-37).
std::string read_series(LineFile &f, Series *s, const std::vector<const char *> &stop, int nvar = 1) {
  std::string line;
  s->nvar = nvar;
  while (f.next(line)) {
    const std::string tok = first_token(line);
    for (const char *w : stop)
      if (same_word(tok, w)) return line;
    char t1[256], t2[256];
    int used = 0;
    if (std::sscanf(line.c_str(), "%255s %255s%n", t1, t2, &used) != 2) f.bad("expected YYYY-MM-DD hh:mm values");
    const char *p = line.c_str() + used;
    for (int k = 0; k < nvar; k++) {
      double v;
      int n = 0;
      if (std::sscanf(p, "%lf%n", &v, &n) != 1) f.bad("expected YYYY-MM-DD hh:mm values");
      s->v.push_back(v);
      p += n;
    }
    bool ok;
    const int64_t t = parse_time(t1, t2, &ok);
    if (!ok) f.bad("bad time stamp");
    s->t.push_back(t);
  }
  return "";
}

// IntrplForc (src/forcing.c:482-531): the reference's bisection for the
// interval that holds t, then linear interpolation between its knots, for
// every variable of the series.
bool interpolate(const Series &s, int64_t t, double *out) {
  const int64_t n = (int64_t)s.t.size();
  if (n < 2 || t < s.t[0] || t > s.t[n - 1]) return false;
  int64_t first = 1, last = n - 1;
  while (first <= last) {
    const int64_t middle = (first + last) / 2;
    if (t >= s.t[middle - 1] && t <= s.t[middle]) {
      const double *a = &s.v[(size_t)(middle - 1) * s.nvar], *b = &s.v[(size_t)middle * s.nvar];
      for (int k = 0; k < s.nvar; k++)
        out[k] = ((double)(s.t[middle] - t) * a[k] + (double)(t - s.t[middle - 1]) * b[k]) /
                 (double)(s.t[middle] - s.t[middle - 1]);
      return true;
    }
    if (s.t[middle] > t)
      last = middle - 1;
    else
      first = middle + 1;
  }
  return false;
}

// Wösten, Lilly, Nemes & Le Bas (1999), "Development and use of a database
// of hydraulic properties of European soils", Geoderma 90: continuous
// pedotransfer functions, used (as ReadSoil does, src/read_soil.c:73-117 and
// src/soil.c:235-314) only for properties the soil file leaves negative.
// silt, clay in %, om in %, bd in g cm-3; topsoil 1 or 0.
double ptf_kv(double silt, double clay, double om, double bd, int top) {
  const double ts = top;
  const double cm_day = std::exp(7.755 + 0.0352 * silt + 0.93 * ts - 0.967 * bd * bd - 0.000484 * clay * clay -
                                 0.000322 * silt * silt + 0.001 / silt - 0.0748 / om - 0.643 * std::log(silt) -
                                 0.01398 * bd * clay - 0.1673 * bd * om + 0.02986 * ts * clay -
                                 0.03305 * ts * silt);
  return cm_day / (100.0 * 24.0 * 3600.0);  // m s-1
}
double ptf_thetas(double silt, double clay, double om, double bd, int top) {
  const double ts = top;
  return 0.7919 + 0.001691 * clay - 0.29619 * bd - 0.000001491 * silt * silt + 0.0000821 * om * om +
         0.02427 / clay + 0.01113 / silt + 0.01472 * std::log(silt) - 0.0000733 * om * clay -
         0.000619 * bd * clay - 0.001183 * bd * om - 0.0001664 * ts * silt;
}
double ptf_thetar(double silt, double clay) { return (clay < 18.0 && 100.0 - silt - clay > 65.0) ? 0.15 : 0.05; }
double ptf_alpha(double silt, double clay, double om, double bd, int top) {
  const double ts = top;
  const double per_cm = std::exp(-14.96 + 0.03135 * clay + 0.0351 * silt + 0.646 * om + 15.29 * bd - 0.192 * ts -
                                 4.671 * bd * bd - 0.000781 * clay * clay - 0.00687 * om * om + 0.0449 / om +
                                 0.0663 * std::log(silt) + 0.1482 * std::log(om) - 0.04546 * bd * silt -
                                 0.4852 * bd * om + 0.00673 * ts * clay);
  return per_cm * 100.0;  // m-1
}
double ptf_beta(double silt, double clay, double om, double bd, int top) {
  const double ts = top;
  return 1.0 + std::exp(-25.23 - 0.02195 * clay + 0.0074 * silt - 0.1940 * om + 45.5 * bd - 7.24 * bd * bd +
                        0.0003658 * clay * clay + 0.002885 * om * om - 12.81 / bd - 0.1524 / silt -
                        0.01958 / om - 0.2876 * std::log(silt) - 0.0709 * std::log(om) - 44.6 * std::log(bd) -
                        0.02264 * bd * clay + 0.0896 * bd * om + 0.00718 * ts * clay);
}

// KrFunc (src/soil.c:8-13): the Mualem-van Genuchten relative conductivity
double kr_func(double beta, double satn) {
  const double a = 1.0 - std::pow(1.0 - std::pow(satn, beta / (beta - 1.0)), (beta - 1.0) / beta);
  return std::sqrt(satn) * a * a;
}

// FieldCapacity (src/soil.c:16-73): the moisture where the conductivity falls
// to 5.79e-9 m s-1 (Chen and Dudhia 2001, with van Genuchten in place of
// Campbell), found by at most 10 Newton steps on the saturation.
double field_capacity(double beta, double kv, double smcmax, double smcmin) {
  const double kfc = 5.79E-9, tol = 1.0E-3;
  const double mx = 1.0 - 1.0 / beta;
  double satn = 0.75, dsatn = 999.0;
  for (int n = 0; n < 10 && dsatn > tol; n++) {
    const double df = kr_func(beta, satn) - kfc / kv;
    const double ftheta = 1.0 - std::pow(satn, 1.0 / mx);
    const double denom = 0.5 * std::pow(satn, -0.5) * std::pow(1.0 - std::pow(ftheta, mx), 2.0) +
                         2.0 * std::pow(satn, 1.0 / mx - 0.5) *
                             (std::pow(ftheta, mx - 1.0) - std::pow(ftheta, 2.0 * mx - 1.0));
    double satnk = satn - df / denom;
    satnk = (satnk > 1.0 - 1.0E-3) ? 1.0 - 1.0E-3 : satnk;
    satnk = (satnk < kSatMin) ? kSatMin : satnk;
    dsatn = std::fabs(satnk - satn);
    satn = satnk;
  }
  if (dsatn > tol) satn = 0.75;
  return (1.0 / 3.0 + 2.0 / 3.0 * satn) * (smcmax - smcmin) + smcmin;
}

// WiltingPoint (src/soil.c:75-81): the moisture at a suction head of 200 m
double wilting_point(double smcmax, double smcmin, double alpha, double beta) {
  const double psiw = 200.0;
  return 0.5 * (smcmax - smcmin) * std::pow(1.0 / (1.0 + std::pow(psiw * alpha, beta)), 1.0 - 1.0 / beta) + smcmin;
}

// RiverEqWid (src/init_river.c:98-124)
double river_eq_width(int order, double depth, double coeff) {
  depth = (depth > 0.0) ? depth : 0.0;
  if (order == kRectangle) return coeff;
  const double e = 1.0 / ((double)order - 1.0);
  return 2.0 * std::pow(depth + kRivDpthMin, e) / std::pow(coeff, e);
}

}  // namespace

struct pihm_deck {
  int32_t ne = 0, nr = 0;
  // element planes, reference order
  std::vector<int32_t> nabr, bc_type;  // [ne*3]
  std::vector<double> area, x, y, zmin, zmax, edge, nabrdist, nabr_x, nabr_y;
  std::vector<double> depth, ksath, ksatv, kinfv, dinf, alpha, beta, porosity, dmac, kmach, kmacv, areafv,
      areafh, rough, rzd;
  // river planes
  std::vector<int32_t> down, leftele, rightele, intrpl_ord, riverbc_type;
  std::vector<double> riv_x, riv_y, riv_area, riv_zmin, riv_zmax, riv_zbed, riv_node_zmax, riv_dist_left,
      riv_dist_right, riv_depth, riv_coeff, riv_length, riv_width, riv_rough, riv_cwr, riv_ksath,
      riv_ksatv, riv_bedthick, riv_porosity;
  pihm_deck_control ctrl{};
  std::vector<double> y0;
  std::vector<double> ic_cmc, ic_sneqv;  // canopy and snow storage at the start
  std::vector<Series> bc, riverbc;
  // land-surface model (include/pihm_land.h): element parameters as
  // InitSoil / InitLc / InitForc leave them, and the forcing series
  std::vector<int32_t> lc_type, meteo_type, lai_type;
  std::vector<double> albedomin, albedomax, shdfac, cmcfactr, cfactr, rgl, rsmin, rsmax, topt, smcmin, smcwlt,
      smcref, zlvl_wind;
  double cal_edir = 1.0, cal_ec = 1.0, cal_ett = 1.0;
  std::vector<Series> meteo, lai;
  std::vector<int32_t> meteo_len, lai_len;  // flattened for pihm_deck_land
  std::vector<int64_t> meteo_time, lai_time;
  std::vector<double> meteo_data, lai_data;
};

namespace {

struct Calib {
  double ksath, ksatv, kinfv, kmach, kmacv, dinf, rzd, dmac, porosity, alpha, beta, areafv, areafh, vegfrac,
      albedo, rough, ec, ett, edir, rivrough, rivksath, rivksatv, rivbedthick, rivdepth, rivshpcoeff, prcp,
      sfctmp;
};

void read_calib(const std::string &path, Calib *c) {
  LineFile f(path);
  c->ksath = keyword_double(f, "KSATH");
  c->ksatv = keyword_double(f, "KSATV");
  c->kinfv = keyword_double(f, "KINF");
  c->kmach = keyword_double(f, "KMACSATH");
  c->kmacv = keyword_double(f, "KMACSATV");
  c->dinf = keyword_double(f, "DINF");
  c->rzd = keyword_double(f, "DROOT");
  c->dmac = keyword_double(f, "DMAC");
  c->porosity = keyword_double(f, "POROSITY");
  c->alpha = keyword_double(f, "ALPHA");
  c->beta = keyword_double(f, "BETA");
  c->areafv = keyword_double(f, "MACVF");
  c->areafh = keyword_double(f, "MACHF");
  c->vegfrac = keyword_double(f, "VEGFRAC");
  c->albedo = keyword_double(f, "ALBEDO");
  c->rough = keyword_double(f, "ROUGH");
  c->ec = keyword_double(f, "EC");
  c->ett = keyword_double(f, "ETT");
  c->edir = keyword_double(f, "EDIR");
  c->rivrough = keyword_double(f, "ROUGH_RIV");
  c->rivksath = keyword_double(f, "KRIVH");
  c->rivksatv = keyword_double(f, "KRIVV");
  c->rivbedthick = keyword_double(f, "BEDTHCK");
  c->rivdepth = keyword_double(f, "RIV_DPTH");
  c->rivshpcoeff = keyword_double(f, "RIV_WDTH");
  // the climate scenario block (src/read_calib.c:140-151)
  std::string line;
  bool found = false;
  while (f.next(line))
    if (same_word(first_token(line), "SCENARIO")) {
      found = true;
      break;
    }
  if (!found) f.bad("expected a SCENARIO block");
  c->prcp = keyword_double(f, "PRCP");
  c->sfctmp = keyword_double(f, "SFCTMP");
}

void read_para(const std::string &path, pihm_deck_control *c) {
  LineFile f(path);
  keyword_int(f, "SIMULATION_MODE");
  c->init_mode = keyword_int(f, "INIT_MODE") > 0 ? 1 : 0;
  keyword_int(f, "ASCII_OUTPUT");
  keyword_int(f, "WATBAL_OUTPUT");
  keyword_int(f, "WRITE_IC");
  c->unsat_mode = keyword_int(f, "UNSAT_MODE");
  c->surf_mode = keyword_int(f, "SURF_MODE");
  c->riv_mode = keyword_int(f, "RIV_MODE");
  c->start = keyword_time(f, "START");
  c->end = keyword_time(f, "END");
  keyword_int(f, "MAX_SPINUP_YEAR");
  const int stepsize = keyword_int(f, "MODEL_STEPSIZE");
  c->lsm_step = keyword_int(f, "LSM_STEP");
  pihm_step_control &s = c->step;
  s.stepsize = stepsize;
  s.abstol = keyword_double(f, "ABSTOL");
  s.reltol = keyword_double(f, "RELTOL");
  s.initstep = keyword_double(f, "INIT_SOLVER_STEP");
  s.nncfn = keyword_double(f, "NUM_NONCOV_FAIL");
  s.nnimax = keyword_double(f, "MAX_NONLIN_ITER");
  s.nnimin = keyword_double(f, "MIN_NONLIN_ITER");
  s.decr = keyword_double(f, "DECR_FACTOR");
  s.incr = keyword_double(f, "INCR_FACTOR");
  s.stmin = keyword_double(f, "MIN_MAXSTEP");
  s.mxstep = 0;
  // print controls (src/read_para.c:96-181): a period word or an interval
  static const char *kPrint[] = {"SURF",    "UNSAT",   "GW",      "RIVSTG",  "RIVGW",   "SNOW",     "CMC",
                                 "INFIL",   "RECHARGE", "EC",     "ETT",     "EDIR",    "RIVFLX0",  "RIVFLX1",
                                 "RIVFLX2", "RIVFLX3", "RIVFLX4", "RIVFLX5", "RIVFLX6", "RIVFLX7",  "RIVFLX8",
                                 "RIVFLX9", "RIVFLX10", "SUBFLX", "SURFFLX", "IC"};
  for (const char *k : kPrint) {
    const std::string line = f.need(k);
    char tok[1024], val[1024];
    if (std::sscanf(line.c_str(), "%1023s %1023s", tok, val) != 2 || !same_word(tok, k))
      f.bad((std::string("expected keyword ") + k).c_str());
    int n;
    if (!same_word(val, "YEARLY") && !same_word(val, "MONTHLY") && !same_word(val, "DAILY") &&
        !same_word(val, "HOURLY") && std::sscanf(val, "%d", &n) != 1)
      f.bad("unknown output control");
  }
  if (c->lsm_step < stepsize || stepsize <= 0 || c->lsm_step % stepsize != 0)
    fail(PIHM_DECK_ERR_VALUE, "%s: LSM_STEP must be an integral multiple of MODEL_STEPSIZE", path.c_str());
}

void build(const std::string &dir, const std::string &project, const std::string &lc_path, int flags,
           pihm_deck *d) {
  const std::string proj = project.substr(0, project.find('.'));
  const std::string base = dir + "/" + proj;

  // ---- .riv: segments, shapes, materials, boundary series (src/read_river.c) ----
  struct Seg {
    int from, to, down, left, right, shp, matl, bc, rsvr;
  };
  std::vector<Seg> seg;
  std::vector<double> shp_depth, shp_coeff, m_rough, m_cwr, m_ksath, m_ksatv, m_bed;
  std::vector<int> shp_ord;
  {
    LineFile f(base + ".riv");
    const int nr = keyword_int(f, "NUMRIV");
    if (nr < 0) f.bad("NUMRIV must not be negative");
    f.need("header");
    seg.resize(nr);
    for (int i = 0; i < nr; i++) {
      const std::string line = f.need("a river segment");
      int index;
      Seg &s = seg[i];
      if (std::sscanf(line.c_str(), "%d %d %d %d %d %d %d %d %d %d", &index, &s.from, &s.to, &s.down, &s.left,
                      &s.right, &s.shp, &s.matl, &s.bc, &s.rsvr) != 10 ||
          index != i + 1)
        f.bad("bad river segment line");
    }
    const int nshp = keyword_int(f, "SHAPE");
    f.need("header");
    for (int i = 0; i < nshp; i++) {
      const std::string line = f.need("a river shape");
      int index, ord;
      double dep, co;
      if (std::sscanf(line.c_str(), "%d %lf %d %lf", &index, &dep, &ord, &co) != 4 || index != i + 1)
        f.bad("bad river shape line");
      shp_depth.push_back(dep);
      shp_ord.push_back(ord);
      shp_coeff.push_back(co);
    }
    const int nmat = keyword_int(f, "MATERIAL");
    f.need("header");
    for (int i = 0; i < nmat; i++) {
      const std::string line = f.need("a river material");
      int index;
      double r, cw, kh, kv, bt;
      if (std::sscanf(line.c_str(), "%d %lf %lf %lf %lf %lf", &index, &r, &cw, &kh, &kv, &bt) != 6 ||
          index != i + 1)
        f.bad("bad river material line");
      m_rough.push_back(r);
      m_cwr.push_back(cw);
      m_ksath.push_back(kh);
      m_ksatv.push_back(kv);
      m_bed.push_back(bt);
    }
    const int nrbc = keyword_int(f, "BC");
    if (nrbc > 0) {
      std::string line = f.need("RIV_TS");
      for (int i = 0; i < nrbc; i++) {
        int index;
        char tok[1024];
        if (std::sscanf(line.c_str(), "%1023s %d", tok, &index) != 2 || !same_word(tok, "RIV_TS") ||
            index != i + 1)
          f.bad("expected RIV_TS block");
        f.need("header");
        f.need("header");
        Series s;
        line = read_series(f, &s, {"RIV_TS", "RES"});
        d->riverbc.push_back(std::move(s));
      }
    }
  }
  const int nr = (int)seg.size();

  // ---- .mesh (src/read_mesh.c) ----
  std::vector<int> node, nabr0;
  std::vector<double> nx, ny, nzmin, nzmax;
  int ne = 0;
  {
    LineFile f(base + ".mesh");
    ne = keyword_int(f, "NUMELE");
    if (ne <= 0) f.bad("NUMELE must be positive");
    f.need("header");
    node.resize(3 * (size_t)ne);
    nabr0.resize(3 * (size_t)ne);
    for (int i = 0; i < ne; i++) {
      const std::string line = f.need("an element");
      int index;
      int *n = &node[3 * (size_t)i], *b = &nabr0[3 * (size_t)i];
      if (std::sscanf(line.c_str(), "%d %d %d %d %d %d %d", &index, &n[0], &n[1], &n[2], &b[0], &b[1], &b[2]) != 7 ||
          index != i + 1)
        f.bad("bad element line");
    }
    const int nn = keyword_int(f, "NUMNODE");
    if (nn <= 0) f.bad("NUMNODE must be positive");
    f.need("header");
    nx.resize(nn);
    ny.resize(nn);
    nzmin.resize(nn);
    nzmax.resize(nn);
    for (int i = 0; i < nn; i++) {
      const std::string line = f.need("a node");
      int index;
      if (std::sscanf(line.c_str(), "%d %lf %lf %lf %lf", &index, &nx[i], &ny[i], &nzmin[i], &nzmax[i]) != 5 ||
          index != i + 1)
        f.bad("bad node line");
    }
  }
  const int nnode = (int)nx.size();
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < kEdges; j++) {
      const int n = node[3 * (size_t)i + j], b = nabr0[3 * (size_t)i + j];
      if (n < 1 || n > nnode) fail(PIHM_DECK_ERR_VALUE, "element %d: node %d out of range", i + 1, n);
      if (b < 0 || b > ne) fail(PIHM_DECK_ERR_VALUE, "element %d: neighbour %d out of range", i + 1, b);
    }

  // ---- .att (src/read_att.c) ----
  std::vector<int> att_soil(ne), att_lc(ne), att_meteo(ne), att_lai(ne), att_bc(3 * (size_t)ne);
  {
    LineFile f(base + ".att");
    f.need("header");
    for (int i = 0; i < ne; i++) {
      const std::string line = f.need("an attribute line");
      int index, geol, source;
      int *b = &att_bc[3 * (size_t)i];
      if (std::sscanf(line.c_str(), "%d %d %d %d %d %d %d %d %d %d", &index, &att_soil[i], &geol, &att_lc[i],
                      &att_meteo[i], &att_lai[i], &source, &b[0], &b[1], &b[2]) != 10)
        f.bad("bad attribute line");
    }
  }

  // ---- .soil (src/read_soil.c) ----
  struct SoilRow {
    double silt, clay, om, bd, kinfv, ksatv, ksath, smcmax, smcmin, alpha, beta, areafh, areafv, dmac, qtz;
    double smcref, smcwlt;  // FieldCapacity and WiltingPoint of the row (src/read_soil.c:118-122)
  };
  std::vector<SoilRow> soil;
  double s_dinf, s_kmacv_ro, s_kmach_ro;
  {
    LineFile f(base + ".soil");
    const int n = keyword_int(f, "NUMSOIL");
    f.need("header");
    soil.resize(n > 0 ? n : 0);
    for (int i = 0; i < n; i++) {
      const std::string line = f.need("a soil type");
      int index;
      SoilRow &r = soil[i];
      if (std::sscanf(line.c_str(), "%d %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", &index,
                      &r.silt, &r.clay, &r.om, &r.bd, &r.kinfv, &r.ksatv, &r.ksath, &r.smcmax, &r.smcmin,
                      &r.alpha, &r.beta, &r.areafh, &r.areafv, &r.dmac, &r.qtz) != 16 ||
          index != i + 1)
        f.bad("bad soil line");
      r.om = (r.om > 0.0) ? r.om : 2.5;
      r.bd = (r.bd > 0.0) ? r.bd : 1.3;
      if (r.kinfv < 0.0) r.kinfv = ptf_kv(r.silt, r.clay, r.om, r.bd, 1);
      if (r.ksatv < 0.0) r.ksatv = ptf_kv(r.silt, r.clay, r.om, r.bd, 0);
      if (r.ksath < 0.0) r.ksath = 10.0 * r.ksatv;
      if (r.smcmax < 0.0) r.smcmax = ptf_thetas(r.silt, r.clay, r.om, r.bd, 0);
      if (r.smcmin < 0.0) r.smcmin = ptf_thetar(r.silt, r.clay);
      if (r.alpha < 0.0) r.alpha = ptf_alpha(r.silt, r.clay, r.om, r.bd, 0);
      if (r.beta < 0.0) r.beta = ptf_beta(r.silt, r.clay, r.om, r.bd, 0);
      r.smcref = field_capacity(r.beta, r.ksatv, r.smcmax, r.smcmin);
      r.smcwlt = wilting_point(r.smcmax, r.smcmin, r.alpha, r.beta);
    }
    s_dinf = keyword_double(f, "DINF");
    s_kmacv_ro = keyword_double(f, "KMACV_RO");
    s_kmach_ro = keyword_double(f, "KMACH_RO");
  }

  // ---- land-cover table (src/read_lc.c) ----
  std::vector<double> lc_rzd, lc_rough;
  std::vector<std::array<double, 15>> lc_row;  // vegfrac rzd rsmin rgl hs snup laimin laimax emissmin emissmax
                                               // albedomin albedomax z0min z0max rough
  double lc_topt, lc_cfactr, lc_rsmax;
  int lc_bare;
  {
    LineFile f(lc_path);
    const int n = keyword_int(f, "NUMLC");
    f.need("header");
    for (int i = 0; i < n; i++) {
      const std::string line = f.need("a land-cover type");
      int index;
      double v[15];
      if (std::sscanf(line.c_str(), "%d %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", &index, &v[0],
                      &v[1], &v[2], &v[3], &v[4], &v[5], &v[6], &v[7], &v[8], &v[9], &v[10], &v[11], &v[12],
                      &v[13], &v[14]) != 16 ||
          index != i + 1)
        f.bad("bad land-cover line");
      lc_rzd.push_back(v[1]);     // vegfrac, rzd, rsmin, ...
      lc_rough.push_back(v[14]);  // ..., z0max, rough
      std::array<double, 15> row;
      std::copy(v, v + 15, row.begin());
      lc_row.push_back(row);
    }
    lc_topt = keyword_double(f, "TOPT_DATA");
    lc_cfactr = keyword_double(f, "CFACTR_DATA");
    lc_rsmax = keyword_double(f, "RSMAX_DATA");
    lc_bare = keyword_int(f, "BARE");
    keyword_int(f, "NATURAL");
  }

  // ---- .meteo (src/read_forc.c): one block per station, "METEO_TS <k>
  // WIND_LVL <m>", two header lines, then time-stamped records of the seven
  // variables; .lai (src/read_lai.c), read when an element names an LAI series ----
  std::vector<double> station_wind;
  {
    LineFile f(base + ".meteo");
    std::string line;
    bool have = f.next(line);
    for (int k = 0; have; k++) {
      int index;
      double zlvl;
      char tok[1024], tok2[1024];
      if (std::sscanf(line.c_str(), "%1023s %d %1023s %lf", tok, &index, tok2, &zlvl) != 4 ||
          !same_word(tok, "METEO_TS") || index != k + 1)
        f.bad("expected METEO_TS <index> WIND_LVL <height>");
      f.need("header");
      f.need("header");
      Series s;
      line = read_series(f, &s, {"METEO_TS"}, PIHM_METEO_NVAR);
      d->meteo.push_back(std::move(s));
      station_wind.push_back(zlvl);
      have = !line.empty();
    }
    if (d->meteo.empty()) f.bad("no METEO_TS block");
  }
  bool any_lai = false;
  for (int v : att_lai) any_lai |= v > 0;
  if (any_lai) {
    LineFile f(base + ".lai");
    std::string line;
    bool have = f.next(line);
    for (int k = 0; have; k++) {
      int index;
      char tok[1024];
      if (std::sscanf(line.c_str(), "%1023s %d", tok, &index) != 2 || !same_word(tok, "LAI_TS") || index != k + 1)
        f.bad("expected LAI_TS <index>");
      f.need("header");
      f.need("header");
      Series s;
      line = read_series(f, &s, {"LAI_TS"}, 1);
      d->lai.push_back(std::move(s));
      have = !line.empty();
    }
  }

  read_para(base + ".para", &d->ctrl);
  Calib cal;
  read_calib(dir + "/" + project + ".calib", &cal);

  // ---- .bc, read when any element edge names a series (src/read_bc.c) ----
  bool any_bc = false;
  for (int v : att_bc) any_bc |= v != 0;
  if (any_bc) {
    LineFile f(base + ".bc");
    std::string line;
    bool have = f.next(line);
    for (int i = 0; have; i++) {
      int index;
      char tok[1024];
      if (std::sscanf(line.c_str(), "%1023s %d", tok, &index) != 2 || !same_word(tok, "BC_TS") ||
          index != i + 1)
        f.bad("expected BC_TS block");
      f.need("header");
      f.need("header");
      Series s;
      line = read_series(f, &s, {"BC_TS"});
      d->bc.push_back(std::move(s));
      have = !line.empty();
    }
  }
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < kEdges; j++) {
      const int b = att_bc[3 * (size_t)i + j];
      if (b != 0 && (b > (int)d->bc.size() || -b > (int)d->bc.size()))
        fail(PIHM_DECK_ERR_VALUE, "element %d: boundary series %d is not in the .bc file", i + 1, b);
    }
  for (int s = 0; s < nr; s++) {
    const int b = seg[s].bc;
    if (b != 0 && (b > (int)d->riverbc.size() || -b > (int)d->riverbc.size()))
      fail(PIHM_DECK_ERR_VALUE, "river segment %d: boundary series %d is not in the .riv file", s + 1, b);
  }

  // ---- InitMesh / InitTopo (src/init_mesh.c, src/init_topo.c:6-52) ----
  d->ne = ne;
  d->nr = nr;
  auto sized = [](std::vector<double> &v, size_t n) { v.assign(n, 0.0); };
  for (auto *v : {&d->area, &d->x, &d->y, &d->zmin, &d->zmax, &d->depth, &d->ksath, &d->ksatv, &d->kinfv,
                  &d->dinf, &d->alpha, &d->beta, &d->porosity, &d->dmac, &d->kmach, &d->kmacv, &d->areafv,
                  &d->areafh, &d->rough, &d->rzd, &d->albedomin, &d->albedomax, &d->shdfac, &d->cmcfactr,
                  &d->cfactr, &d->rgl, &d->rsmin, &d->rsmax, &d->topt, &d->smcmin, &d->smcwlt, &d->smcref,
                  &d->zlvl_wind})
    sized(*v, ne);
  d->lc_type.assign(ne, 0);
  d->meteo_type.assign(ne, 0);
  d->lai_type.assign(ne, 0);
  for (auto *v : {&d->edge, &d->nabrdist, &d->nabr_x, &d->nabr_y}) sized(*v, 3 * (size_t)ne);
  d->nabr.assign(nabr0.begin(), nabr0.end());
  d->bc_type.assign(att_bc.begin(), att_bc.end());
  auto nodexy = [&](int i, double *x, double *y, double *zn, double *zx) {
    for (int j = 0; j < kEdges; j++) {
      const int n = node[3 * (size_t)i + j] - 1;
      x[j] = nx[n];
      y[j] = ny[n];
      if (zn) zn[j] = nzmin[n];
      if (zx) zx[j] = nzmax[n];
    }
  };
  for (int i = 0; i < ne; i++) {
    double x[3], y[3], zn[3], zx[3];
    nodexy(i, x, y, zn, zx);
    d->area[i] = 0.5 * ((x[1] - x[0]) * (y[2] - y[0]) - (y[1] - y[0]) * (x[2] - x[0]));
    d->x[i] = (x[0] + x[1] + x[2]) / 3.0;
    d->y[i] = (y[0] + y[1] + y[2]) / 3.0;
    d->zmin[i] = (zn[0] + zn[1] + zn[2]) / 3.0;
    d->zmax[i] = (zx[0] + zx[1] + zx[2]) / 3.0;
    const double e0x = x[1] - x[2], e0y = y[1] - y[2], e1x = x[2] - x[0], e1y = y[2] - y[0];
    const double e2x = x[0] - x[1], e2y = y[0] - y[1];
    d->edge[3 * (size_t)i] = std::sqrt(e0x * e0x + e0y * e0y);
    d->edge[3 * (size_t)i + 1] = std::sqrt(e1x * e1x + e1y * e1y);
    d->edge[3 * (size_t)i + 2] = std::sqrt(e2x * e2x + e2y * e2y);
  }

  // ---- InitSoil (src/init_soil.c) and InitLc (src/init_lc.c) ----
  for (int i = 0; i < ne; i++) {
    const int st = att_soil[i] - 1, lt = att_lc[i] - 1;
    if (st < 0 || st >= (int)soil.size()) fail(PIHM_DECK_ERR_VALUE, "element %d: soil type %d undefined", i + 1, st + 1);
    if (lt < 0 || lt >= (int)lc_rough.size())
      fail(PIHM_DECK_ERR_VALUE, "element %d: land-cover type %d undefined", i + 1, lt + 1);
    const SoilRow &r = soil[st];
    d->dinf[i] = cal.dinf * s_dinf;
    d->depth[i] = d->zmax[i] - d->zmin[i];
    d->ksath[i] = cal.ksath * r.ksath;
    d->ksatv[i] = cal.ksatv * r.ksatv;
    d->kinfv[i] = cal.kinfv * r.kinfv;
    const double smcmin = cal.porosity * r.smcmin, smcmax = cal.porosity * r.smcmax;
    d->porosity[i] = smcmax - smcmin;
    if (d->porosity[i] > 1.0 || d->porosity[i] <= 0.0)
      fail(PIHM_DECK_ERR_VALUE, "element %d: porosity %g out of (0, 1]", i + 1, d->porosity[i]);
    d->alpha[i] = cal.alpha * r.alpha;
    d->beta[i] = cal.beta * r.beta;
    d->dmac[i] = cal.dmac * r.dmac;
    d->dmac[i] = (d->dmac[i] > d->depth[i]) ? d->depth[i] : d->dmac[i];
    d->areafh[i] = cal.areafh * r.areafh;
    d->areafv[i] = cal.areafv * r.areafv;
    d->kmacv[i] = cal.kmacv * s_kmacv_ro * r.kinfv;
    d->kmach[i] = cal.kmach * s_kmach_ro * r.ksath;
    d->rzd[i] = cal.rzd * lc_rzd[lt];
    d->rough[i] = cal.rough * lc_rough[lt];
    // the land-surface model's soil and land-cover parameters
    // (src/init_soil.c:34-54, src/init_lc.c:19-38 without the Noah factors)
    d->smcmin[i] = smcmin;
    d->smcwlt[i] = cal.porosity * r.smcwlt;
    d->smcref[i] = cal.porosity * r.smcref;
    const std::array<double, 15> &row = lc_row[lt];
    d->rsmin[i] = row[2];
    d->rgl[i] = row[3];
    d->rsmax[i] = lc_rsmax;
    d->topt[i] = lc_topt;
    d->shdfac[i] = cal.vegfrac * row[0];
    d->albedomin[i] = cal.albedo * row[10];
    d->albedomax[i] = cal.albedo * row[11];
    d->cmcfactr[i] = kCmcFactr;
    d->cfactr[i] = lc_cfactr;
    if (lc_bare == att_lc[i]) d->shdfac[i] = 0.0;
    d->lc_type[i] = att_lc[i];
    d->meteo_type[i] = att_meteo[i];
    d->lai_type[i] = att_lai[i];
    if (att_meteo[i] < 1 || att_meteo[i] > (int)d->meteo.size())
      fail(PIHM_DECK_ERR_VALUE, "element %d: meteorological station %d is not in the .meteo file", i + 1, att_meteo[i]);
    if (att_lai[i] < 0 || att_lai[i] > (int)d->lai.size())
      fail(PIHM_DECK_ERR_VALUE, "element %d: LAI series %d is not in the .lai file", i + 1, att_lai[i]);
    d->zlvl_wind[i] = station_wind[att_meteo[i] - 1];
  }
  // InitForc's climate scenario (src/init_forc.c:8-17)
  for (Series &s : d->meteo)
    for (size_t j = 0; j < s.t.size(); j++) {
      s.v[j * PIHM_METEO_NVAR + PIHM_METEO_PRCP] *= cal.prcp;
      s.v[j * PIHM_METEO_NVAR + PIHM_METEO_SFCTMP] += cal.sfctmp;
    }
  d->cal_edir = cal.edir;
  d->cal_ec = cal.ec;
  d->cal_ett = cal.ett;
  auto flatten = [](const std::vector<Series> &ss, std::vector<int32_t> *len, std::vector<int64_t> *tt,
                    std::vector<double> *vv) {
    for (const Series &s : ss) {
      len->push_back((int32_t)s.t.size());
      tt->insert(tt->end(), s.t.begin(), s.t.end());
      vv->insert(vv->end(), s.v.begin(), s.v.end());
    }
  };
  flatten(d->meteo, &d->meteo_len, &d->meteo_time, &d->meteo_data);
  flatten(d->lai, &d->lai_len, &d->lai_time, &d->lai_data);

  // ---- InitRiver (src/init_river.c:6-96) ----
  for (auto *v : {&d->riv_x, &d->riv_y, &d->riv_area, &d->riv_zmin, &d->riv_zmax, &d->riv_zbed, &d->riv_node_zmax,
                  &d->riv_dist_left, &d->riv_dist_right, &d->riv_depth, &d->riv_coeff, &d->riv_length,
                  &d->riv_width, &d->riv_rough, &d->riv_cwr, &d->riv_ksath, &d->riv_ksatv, &d->riv_bedthick,
                  &d->riv_porosity})
    sized(*v, nr);
  d->down.resize(nr);
  d->leftele.resize(nr);
  d->rightele.resize(nr);
  d->intrpl_ord.resize(nr);
  d->riverbc_type.resize(nr);
  for (int s = 0; s < nr; s++) {
    const Seg &g = seg[s];
    if (g.left < 1 || g.left > ne || g.right < 1 || g.right > ne)
      fail(PIHM_DECK_ERR_VALUE, "river segment %d: bank element out of range", s + 1);
    if (g.from < 1 || g.from > nnode || g.to < 1 || g.to > nnode)
      fail(PIHM_DECK_ERR_VALUE, "river segment %d: node out of range", s + 1);
    if (g.shp < 1 || g.shp > (int)shp_depth.size() || g.matl < 1 || g.matl > (int)m_rough.size())
      fail(PIHM_DECK_ERR_VALUE, "river segment %d: shape or material undefined", s + 1);
    if (g.down == 0 || g.down > nr) fail(PIHM_DECK_ERR_VALUE, "river segment %d: bad downstream %d", s + 1, g.down);
    const int L = g.left - 1, R = g.right - 1, F = g.from - 1, T = g.to - 1;
    d->down[s] = g.down;
    d->leftele[s] = g.left;
    d->rightele[s] = g.right;
    d->riverbc_type[s] = g.bc;
    for (int j = 0; j < kEdges; j++) {
      if (d->nabr[3 * (size_t)L + j] == g.right) d->nabr[3 * (size_t)L + j] = -(s + 1);
      if (d->nabr[3 * (size_t)R + j] == g.left) d->nabr[3 * (size_t)R + j] = -(s + 1);
    }
    d->riv_x[s] = 0.5 * (nx[F] + nx[T]);
    d->riv_y[s] = 0.5 * (ny[F] + ny[T]);
    d->riv_zmax[s] = 0.5 * (nzmax[F] + nzmax[T]);
    d->riv_zmin[s] = d->riv_zmax[s] - (0.5 * (d->zmax[L] + d->zmax[R]) - 0.5 * (d->zmin[L] + d->zmin[R]));
    d->riv_node_zmax[s] = nzmax[T];
    const double dlx = d->riv_x[s] - d->x[L], dly = d->riv_y[s] - d->y[L];
    const double drx = d->riv_x[s] - d->x[R], dry = d->riv_y[s] - d->y[R];
    d->riv_dist_left[s] = std::sqrt(dlx * dlx + dly * dly);
    d->riv_dist_right[s] = std::sqrt(drx * drx + dry * dry);
    d->riv_depth[s] = cal.rivdepth * shp_depth[g.shp - 1];
    d->intrpl_ord[s] = shp_ord[g.shp - 1];
    if (d->intrpl_ord[s] < kRectangle || d->intrpl_ord[s] > kCubic)
      fail(PIHM_DECK_ERR_VALUE, "river shape %d: interpolation order %d undefined", g.shp, d->intrpl_ord[s]);
    d->riv_coeff[s] = cal.rivshpcoeff * shp_coeff[g.shp - 1];
    const double lx = nx[F] - nx[T], ly = ny[F] - ny[T];
    d->riv_length[s] = std::sqrt(lx * lx + ly * ly);
    d->riv_width[s] = river_eq_width(d->intrpl_ord[s], d->riv_depth[s], d->riv_coeff[s]);
    d->riv_zbed[s] = d->riv_zmax[s] - d->riv_depth[s];
    d->riv_rough[s] = cal.rivrough * m_rough[g.matl - 1];
    d->riv_cwr[s] = m_cwr[g.matl - 1];
    d->riv_ksath[s] = cal.rivksath * m_ksath[g.matl - 1];
    d->riv_ksatv[s] = cal.rivksatv * m_ksatv[g.matl - 1];
    d->riv_bedthick[s] = cal.rivbedthick * m_bed[g.matl - 1];
    d->riv_porosity[s] = 0.5 * (d->porosity[L] + d->porosity[R]);
    d->riv_area[s] = d->riv_length[s] * river_eq_width(d->intrpl_ord[s], d->riv_depth[s], d->riv_coeff[s]);
  }

  // ---- CorrElev (src/initialize.c:225-383), when asked ----
  if (flags & PIHM_DECK_CORR_ELEV) {
    for (int i = 0; i < ne; i++) {
      bool sink = true;
      for (int j = 0; j < kEdges && sink; j++) {
        const int b = d->nabr[3 * (size_t)i + j];
        if (b == 0) continue;
        const double nz = (b > 0) ? d->zmax[b - 1] : d->riv_zmax[-b - 1];
        if (d->zmax[i] >= nz) sink = false;
      }
      if (!sink) continue;
      double lowest = 1.0e7;
      for (int j = 0; j < kEdges; j++) {
        const int b = d->nabr[3 * (size_t)i + j];
        if (b == 0) continue;
        const double nz = (b > 0) ? d->zmax[b - 1] : d->riv_zmax[-b - 1];
        lowest = (nz < lowest) ? nz : lowest;
      }
      d->zmin[i] += (lowest - d->zmax[i]);
      d->zmax[i] = lowest;
    }
  }

  // ---- InitSurfL (src/initialize.c:385-458) ----
  for (int i = 0; i < ne; i++) {
    double x[3], y[3];
    nodexy(i, x, y, nullptr, nullptr);
    for (int j = 0; j < kEdges; j++) {
      const int a = (j + 1) % 3, b = (j + 2) % 3;  // the edge opposite node j
      const double distx = d->x[i] - 0.5 * (x[a] + x[b]);
      const double disty = d->y[i] - 0.5 * (y[a] + y[b]);
      const size_t k = 3 * (size_t)i + j;
      const int nb = d->nabr[k];
      if (nb == 0) {
        d->nabr_x[k] = d->x[i] - 2.0 * distx;
        d->nabr_y[k] = d->y[i] - 2.0 * disty;
        const double circ = d->edge[3 * (size_t)i] * d->edge[3 * (size_t)i + 1] * d->edge[3 * (size_t)i + 2] /
                            (4.0 * d->area[i]);
        const double half = d->edge[k] / 2.0;
        d->nabrdist[k] = std::sqrt(circ * circ - half * half);
      } else {
        d->nabr_x[k] = (nb > 0) ? d->x[nb - 1] : d->riv_x[-nb - 1];
        d->nabr_y[k] = (nb > 0) ? d->y[nb - 1] : d->riv_y[-nb - 1];
        double dist = (d->x[i] - d->nabr_x[k]) * (d->x[i] - d->nabr_x[k]);
        dist += (d->y[i] - d->nabr_y[k]) * (d->y[i] - d->nabr_y[k]);
        d->nabrdist[k] = std::sqrt(dist);
      }
    }
  }

  // ---- initial state: RelaxIc (src/initialize.c:496-575) or the restart file ----
  d->y0.assign(3 * (size_t)ne + 2 * (size_t)nr, 0.0);
  d->ic_cmc.assign(ne, 0.0);  // RelaxIc (src/initialize.c:509-510)
  d->ic_sneqv.assign(ne, 0.0);
  if (d->ctrl.init_mode == 0) {
    const double kInitUnsat = 0.1;
    for (int i = 0; i < ne; i++) {
      d->y0[i] = 0.0;
      d->y0[(size_t)ne + i] = kInitUnsat;
      d->y0[2 * (size_t)ne + i] = d->depth[i] - kInitUnsat;
    }
    for (int s = 0; s < nr; s++) {
      d->y0[3 * (size_t)ne + s] = 0.0;
      d->y0[3 * (size_t)ne + nr + s] = d->riv_zbed[s] - d->riv_zmin[s] - 0.1;
    }
  } else {
    const std::string ic = dir + "/" + project + ".ic";
    const int rc = pihm_ic_read(ic.c_str(), ne, nr, d->y0.data(), d->ic_cmc.data(), d->ic_sneqv.data());
    if (rc != 0) fail(rc == PIHM_DECK_ERR_IO ? rc : PIHM_DECK_ERR_IO, "cannot read restart file %s", ic.c_str());
  }
}

}  // namespace

extern "C" {

int pihm_deck_read(const char *dir, const char *project, const char *lc_table, int flags, pihm_deck **out) {
  if (!dir || !project || !out) {
    g_error = "null argument";
    return PIHM_GPU_ERR_ARG;
  }
  *out = nullptr;
  auto d = std::make_unique<pihm_deck>();
  const std::string lc = lc_table ? std::string(lc_table) : std::string(dir) + "/../vegprmt.tbl";
  try {
    build(dir, project, lc, flags, d.get());
  } catch (const DeckError &e) {
    return e.code;
  } catch (const std::bad_alloc &) {
    g_error = "out of memory";
    return PIHM_GPU_ERR_NOMEM;
  }
  g_error.clear();
  *out = d.release();
  return PIHM_GPU_OK;
}

const char *pihm_deck_error(void) { return g_error.c_str(); }

void pihm_deck_free(pihm_deck *d) { delete d; }

int pihm_deck_mesh(const pihm_deck *d, pihm_gpu_mesh *m) {
  if (!d || !m) return PIHM_GPU_ERR_ARG;
  *m = pihm_gpu_mesh{};
  m->nelem = d->ne;
  m->nriver = d->nr;
  m->nabr = d->nabr.data();
  m->bc_type = d->bc_type.data();
  m->area = d->area.data();
  m->zmin = d->zmin.data();
  m->zmax = d->zmax.data();
  m->edge = d->edge.data();
  m->nabrdist = d->nabrdist.data();
  m->nabr_x = d->nabr_x.data();
  m->nabr_y = d->nabr_y.data();
  m->depth = d->depth.data();
  m->ksath = d->ksath.data();
  m->ksatv = d->ksatv.data();
  m->kinfv = d->kinfv.data();
  m->dinf = d->dinf.data();
  m->alpha = d->alpha.data();
  m->beta = d->beta.data();
  m->porosity = d->porosity.data();
  m->dmac = d->dmac.data();
  m->kmach = d->kmach.data();
  m->kmacv = d->kmacv.data();
  m->areafv = d->areafv.data();
  m->areafh = d->areafh.data();
  m->rough = d->rough.data();
  m->rzd = d->rzd.data();
  m->down = d->down.data();
  m->leftele = d->leftele.data();
  m->rightele = d->rightele.data();
  m->intrpl_ord = d->intrpl_ord.data();
  m->riverbc_type = d->riverbc_type.data();
  m->riv_area = d->riv_area.data();
  m->riv_zmin = d->riv_zmin.data();
  m->riv_zmax = d->riv_zmax.data();
  m->riv_zbed = d->riv_zbed.data();
  m->riv_node_zmax = d->riv_node_zmax.data();
  m->riv_dist_left = d->riv_dist_left.data();
  m->riv_dist_right = d->riv_dist_right.data();
  m->riv_depth = d->riv_depth.data();
  m->riv_coeff = d->riv_coeff.data();
  m->riv_length = d->riv_length.data();
  m->riv_width = d->riv_width.data();
  m->riv_rough = d->riv_rough.data();
  m->riv_cwr = d->riv_cwr.data();
  m->riv_ksath = d->riv_ksath.data();
  m->riv_ksatv = d->riv_ksatv.data();
  m->riv_bedthick = d->riv_bedthick.data();
  m->riv_porosity = d->riv_porosity.data();
  return PIHM_GPU_OK;
}

int pihm_deck_control_get(const pihm_deck *d, pihm_deck_control *c) {
  if (!d || !c) return PIHM_GPU_ERR_ARG;
  *c = d->ctrl;
  return PIHM_GPU_OK;
}

int pihm_deck_initial_state(const pihm_deck *d, double *y0) {
  if (!d || !y0) return PIHM_GPU_ERR_ARG;
  std::memcpy(y0, d->y0.data(), sizeof(double) * d->y0.size());
  return PIHM_GPU_OK;
}

int pihm_deck_initial_storage(const pihm_deck *d, double *cmc, double *sneqv) {
  if (!d) return PIHM_GPU_ERR_ARG;
  if (cmc) std::memcpy(cmc, d->ic_cmc.data(), sizeof(double) * d->ic_cmc.size());
  if (sneqv) std::memcpy(sneqv, d->ic_sneqv.data(), sizeof(double) * d->ic_sneqv.size());
  return PIHM_GPU_OK;
}

int pihm_deck_land(const pihm_deck *d, pihm_land_params *p, pihm_forcing_series *s) {
  if (!d || !p || !s) return PIHM_GPU_ERR_ARG;
  *p = pihm_land_params{};
  p->nelem = d->ne;
  p->lc_type = d->lc_type.data();
  p->meteo_type = d->meteo_type.data();
  p->lai_type = d->lai_type.data();
  p->albedomin = d->albedomin.data();
  p->albedomax = d->albedomax.data();
  p->shdfac = d->shdfac.data();
  p->cmcfactr = d->cmcfactr.data();
  p->cfactr = d->cfactr.data();
  p->rgl = d->rgl.data();
  p->rsmin = d->rsmin.data();
  p->rsmax = d->rsmax.data();
  p->topt = d->topt.data();
  p->smcmin = d->smcmin.data();
  p->smcwlt = d->smcwlt.data();
  p->smcref = d->smcref.data();
  p->zlvl_wind = d->zlvl_wind.data();
  p->cal_edir = d->cal_edir;
  p->cal_ec = d->cal_ec;
  p->cal_ett = d->cal_ett;
  *s = pihm_forcing_series{};
  s->nmeteo = (int32_t)d->meteo.size();
  s->meteo_len = d->meteo_len.data();
  s->meteo_time = d->meteo_time.data();
  s->meteo_data = d->meteo_data.data();
  s->nlai = (int32_t)d->lai.size();
  s->lai_len = d->lai_len.data();
  s->lai_time = d->lai_time.data();
  s->lai_data = d->lai_data.data();
  return PIHM_GPU_OK;
}

int pihm_deck_bc(const pihm_deck *d, int64_t t, double *elem_bc, double *river_bc) {
  if (!d) return PIHM_GPU_ERR_ARG;
  std::vector<double> ev(d->bc.size()), rv(d->riverbc.size());
  for (size_t k = 0; k < d->bc.size(); k++)
    if (!interpolate(d->bc[k], t, &ev[k])) {
      g_error = "time outside element boundary series " + std::to_string(k + 1);
      return PIHM_DECK_ERR_VALUE;
    }
  for (size_t k = 0; k < d->riverbc.size(); k++)
    if (!interpolate(d->riverbc[k], t, &rv[k])) {
      g_error = "time outside river boundary series " + std::to_string(k + 1);
      return PIHM_DECK_ERR_VALUE;
    }
  if (elem_bc)
    for (size_t k = 0; k < d->bc_type.size(); k++) {
      const int b = d->bc_type[k];
      elem_bc[k] = b > 0 ? ev[b - 1] : (b < 0 ? ev[-b - 1] : 0.0);
    }
  if (river_bc)
    for (int s = 0; s < d->nr; s++) {
      const int b = d->riverbc_type[s];
      river_bc[s] = b > 0 ? rv[b - 1] : (b < 0 ? rv[-b - 1] : 0.0);
    }
  return PIHM_GPU_OK;
}

}  // extern "C"
