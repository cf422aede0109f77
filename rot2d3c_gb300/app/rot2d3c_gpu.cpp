// Main program of a run on one GPU over the C-ABI (include/r2d3c.h): the
// control flow of PROGRAM Rot2D3C (src/Rot2D3C.para.f90:2-639) with the
// reference's inputs, output cadence, file names and formats.
//
//   rot2d3c_gpu --n N [--dir RUNDIR] [--fp32] [--max-steps K]
//
// Reads parameter.inp (25 values read positionally, list-directed, then the
// input and output directories, :134-163) and status.inp (:125-130) from
// RUNDIR; builds the initial condition (stat == 0, :245-299) or reads the
// binary fields of output `stat` (:300-338); sets up the forcing (:343-381);
// runs the main loop (:393-615): cond_check every cstep steps into
// energy_bal.txt, enstrophy_bal.txt, helicity_bal.txt, max_min.txt
// (E23.14E3), spectrum/transfers every sstep steps into
// odir/spectrum|transfer|fluxes.XXXX.txt (E24.15E3) and time_spec.txt
// (A4,F12.6), binary fields every tstep steps into
// odir/ps|vz|ww|invlap_psi.000.XXX.out (one sequential unformatted record,
// 4-byte markers) and time_field.txt (A3,F12.6).  Between outputs, whole
// stretches of steps go to r2d3c_advance (CFL dt, forcing, RK step replayed
// from one CUDA graph).  The grid size is a run-time value (fixed at compile
// time in the reference, pseudospec2D_mod.f90:7-14).
#include <cerrno>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/r2d3c.h"

namespace {

struct Failure : std::runtime_error {
  using std::runtime_error::runtime_error;
};

void check(int rc, const char* where) {
  if (rc != R2D3C_OK) throw Failure(std::string(where) + ": " + r2d3c_last_error());
}

// ---------------------------------------------------------------- inputs
// The value a list-directed READ of one item takes from a record: the first
// token before a blank, comma or slash; Fortran 'd' exponents accepted.
std::string first_value(const std::string& line) {
  std::string s = line;
  for (char& c : s)
    if (c == ',') c = ' ';
  std::istringstream is(s);
  std::string tok;
  if (!(is >> tok)) throw Failure("empty record where a value was expected");
  const size_t slash = tok.find('/');
  if (slash != std::string::npos) tok = tok.substr(0, slash);
  for (char& c : tok)
    if (c == 'd' || c == 'D') c = 'e';
  return tok;
}
double as_double(const std::string& tok) {
  char* end = nullptr;
  errno = 0;
  const double v = std::strtod(tok.c_str(), &end);
  if (errno || end == tok.c_str() || *end) throw Failure("not a number: " + tok);
  return v;
}
int as_int(const std::string& tok) {
  char* end = nullptr;
  errno = 0;
  const long v = std::strtol(tok.c_str(), &end, 10);
  if (errno || end == tok.c_str() || *end) throw Failure("not an integer: " + tok);
  return (int)v;
}

std::vector<std::string> read_lines(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw Failure("cannot open " + path);
  std::vector<std::string> out;
  std::string l;
  while (std::getline(f, l)) out.push_back(l);
  return out;
}

std::string rtrim(std::string s) {
  while (!s.empty() && (s.back() == ' ' || s.back() == '\r' || s.back() == '\t')) s.pop_back();
  return s;
}

struct Inputs {
  r2d3c_params p{};
  std::string idir, odir;
  int stat = 0;
  double time = 0.0;
};

Inputs read_inputs(const std::string& dir, int n) {
  Inputs in;
  const std::vector<std::string> L = read_lines(dir + "/parameter.inp");
  if (L.size() < 27) throw Failure(dir + "/parameter.inp: expected 27 records");
  r2d3c_params& p = in.p;
  p.n = n;
  int i = 0;
  auto D = [&]() { return as_double(first_value(L[i++])); };
  auto I = [&]() { return as_int(first_value(L[i++])); };
  p.cfl = D();  // record order of Rot2D3C.para.f90:136-160
  p.step = I();
  p.cstep = I();
  p.sstep = I();
  p.tstep = I();
  p.fp0 = D();
  p.fz0 = D();
  p.u0 = D();
  p.v0 = D();
  p.kdn = D();
  p.kup = D();
  p.nu = D();
  p.hnu = D();
  p.nn = I();
  p.mm = I();
  p.nuv = D();
  p.hnuv = D();
  p.nnv = I();
  p.mmv = I();
  p.omega = D();
  p.seed = I();
  p.iflow = I();
  p.prm1 = D();
  p.prm2 = D();
  p.dt_corr = D();
  in.idir = dir + "/" + rtrim(L[25].substr(0, 100));
  in.odir = dir + "/" + rtrim(L[26].substr(0, 100));
  const std::vector<std::string> S = read_lines(dir + "/status.inp");
  if (S.size() < 2) throw Failure(dir + "/status.inp: expected 2 records");
  in.stat = as_int(first_value(S[0]));
  in.time = as_double(first_value(S[1]));
  return in;
}

// --------------------------------------------------------------- formats
// Fortran Ew.dEe as gfortran writes it: 0.d1..dd E sign eee, right-aligned.
// The d significant digits are printf's %.{d-1}e digits (correctly rounded,
// ties to even, from the exact binary value); only the layout differs.
std::string fortran_e(double x, int w, int d, int e = 3) {
  std::string s;
  if (std::isnan(x)) {
    s = "NaN";
  } else if (std::isinf(x)) {
    s = x < 0 ? "-Infinity" : "Infinity";
  } else {
    const bool neg = std::signbit(x);
    std::string body;
    if (x == 0.0) {
      body = "0." + std::string(d, '0') + "E+" + std::string(e, '0');
    } else {
      char buf[64];
      std::snprintf(buf, sizeof buf, "%.*e", d - 1, std::fabs(x));  // "D.DDDDe+XX"
      const char* ep = std::strchr(buf, 'e');
      const int ex = std::atoi(ep + 1) + 1;
      std::string digits;
      for (const char* c = buf; c < ep; ++c)
        if (*c != '.') digits += *c;
      char eb[16];
      std::snprintf(eb, sizeof eb, "%0*d", e, ex < 0 ? -ex : ex);
      body = "0." + digits + "E" + (ex < 0 ? "-" : "+") + eb;
    }
    s = (neg ? "-" : "") + body;
  }
  if ((int)s.size() > w) return std::string(w, '*');
  return std::string(w - s.size(), ' ') + s;
}

// Fortran Fw.d (non-negative widths; the optional leading zero dropped when
// the value would not fit otherwise)
std::string fortran_f(double x, int w, int d) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*f", d, x);
  std::string s = buf;
  if ((int)s.size() > w && s.rfind("0.", 0) == 0) s = s.substr(1);
  if ((int)s.size() > w && s.rfind("-0.", 0) == 0) s = "-" + s.substr(2);
  if ((int)s.size() > w) return std::string(w, '*');
  return std::string(w - s.size(), ' ') + s;
}

void append_line(const std::string& path, const std::string& line) {
  std::FILE* f = std::fopen(path.c_str(), "a");
  if (!f) throw Failure("cannot open " + path);
  std::fputs(line.c_str(), f);
  std::fputc('\n', f);
  std::fclose(f);
}

void write_text(const std::string& path, const std::vector<std::string>& lines) {
  std::FILE* f = std::fopen(path.c_str(), "w");
  if (!f) throw Failure("cannot open " + path);
  for (const std::string& l : lines) {
    std::fputs(l.c_str(), f);
    std::fputc('\n', f);
  }
  std::fclose(f);
}

// one sequential unformatted record of REAL*8 R(n,n) with 4-byte markers
void write_field(const std::string& path, const std::vector<double>& r) {
  const uint64_t bytes = r.size() * sizeof(double);
  if (bytes > 0x7FFFFFFFull) throw Failure("record larger than 2 GiB needs gfortran subrecords");
  const int32_t mark = (int32_t)bytes;
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw Failure("cannot open " + path);
  bool ok = std::fwrite(&mark, 4, 1, f) == 1 && std::fwrite(r.data(), 1, bytes, f) == bytes &&
            std::fwrite(&mark, 4, 1, f) == 1;
  ok = std::fclose(f) == 0 && ok;
  if (!ok) throw Failure("write failed: " + path);
}

std::vector<double> read_field(const std::string& path, int n) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw Failure("cannot open " + path);
  const uint64_t want = (uint64_t)n * n * sizeof(double);
  std::vector<double> r((size_t)n * n);
  int32_t head = 0, tail = 0;
  bool ok = std::fread(&head, 4, 1, f) == 1 && std::fread(r.data(), 1, want, f) == want &&
            std::fread(&tail, 4, 1, f) == 1;
  std::fclose(f);
  if (!ok || (uint64_t)head != want || (uint64_t)tail != want)
    throw Failure(path + ": not one record of " + std::to_string(want) + " bytes");
  return r;
}

// character counters c//d//u of a 3-digit output index (:91-97, :315-320)
void digits3(int v, int& ic, int& id, int& iu) {
  const float f = (float)v;
  ic = 48 + (int)(f / 100.0f);
  id = 48 + (int)(f / 10.0f) - (int)(f / 100.0f) * 10;
  iu = 48 + v - (int)(f / 10.0f) * 10;
}

// ------------------------------------------------------------------ run
struct Run {
  int n;
  std::string dir;
  Inputs in;
  r2d3c_ctx* ctx = nullptr;
  int seed = 0, seed1 = 0;
  int ini = 1, timet = 0, timec = 0, times = 0;
  int ic = 48, id = 48, iu = 48, jt = 48, jc = 48, jd = 48, ju = 48;
  double time = 0.0;
  const std::string node = "000";  // one rank (:91-97)

  Run(int n_, const std::string& d, int precision) : n(n_), dir(d) {
    in = read_inputs(dir, n);
    check(r2d3c_create(&in.p, precision, &ctx), "r2d3c_create");
    seed = in.p.seed;
    time = in.time;
  }
  ~Run() {
    if (ctx) r2d3c_destroy(ctx);
  }

  void setup() {
    const r2d3c_params& p = in.p;
    if (in.stat == 0) {  // :245-299
      ini = 1;
      timet = p.tstep;
      timec = p.cstep;
      times = p.sstep;
      check(r2d3c_initial_conditions(ctx, &seed), "r2d3c_initial_conditions");
    } else {  // :300-338
      ini = (int)((in.stat - 1) * p.tstep);
      const double dump = (double)ini / (double)p.sstep + 1;
      timet = timec = times = 0;
      jt = 48 + (int)(dump / 1000);
      jc = 48 + (int)(dump / 100) - (int)(dump / 1000) * 10;
      jd = 48 + (int)(dump / 10) - (int)(dump / 100) * 10;
      ju = 48 + (int)dump - (int)(dump / 10) * 10;
      digits3(in.stat, ic, id, iu);
      const std::string ext = {(char)ic, (char)id, (char)iu};
      const std::vector<double> a = read_field(in.idir + "/ps." + node + "." + ext + ".out", n);
      const std::vector<double> b = read_field(in.idir + "/vz." + node + "." + ext + ".out", n);
      check(r2d3c_set_state_physical(ctx, a.data(), b.data()), "r2d3c_set_state_physical");
    }
    check(r2d3c_forcing_init(ctx, &seed, &seed1), "r2d3c_forcing_init");  // :343-381
    check(r2d3c_set_time(ctx, time), "r2d3c_set_time");
  }

  void cond_check() {  // :410, pseudospec2D_Rot2D3C.f90:592-609
    double out[30];
    check(r2d3c_cond_check(ctx, time, out), "r2d3c_cond_check");
    const char* names[4] = {"energy_bal.txt", "enstrophy_bal.txt", "helicity_bal.txt", "max_min.txt"};
    const int lo[5] = {0, 12, 17, 25, 30};
    for (int f = 0; f < 4; ++f) {
      std::string line;
      for (int k = lo[f]; k < lo[f + 1]; ++k) line += fortran_e(out[k], 23, 14);
      append_line(dir + "/" + names[f], line);
    }
  }

  void spectra() {  // :428-457
    if (++ju == 58) {
      ju = 48;
      ++jd;
    }
    if (jd == 58) {
      jd = 48;
      ++jc;
    }
    if (jc == 58) {
      jc = 48;
      ++jt;
    }
    const std::string ext4 = {(char)jt, (char)jc, (char)jd, (char)ju};
    const int nb = n / 2 + 1;
    std::vector<double> ek(nb), ezk(nb), f0(nb), f1(nb), f2(nb);
    check(r2d3c_spectrum(ctx, ek.data(), ezk.data()), "r2d3c_spectrum");
    std::vector<std::string> L;
    for (int k = 0; k < nb; ++k) L.push_back(fortran_e(ek[k], 24, 15) + fortran_e(ezk[k], 24, 15));
    write_text(in.odir + "/spectrum." + ext4 + ".txt", L);
    check(r2d3c_transfers(ctx, f0.data(), f1.data(), f2.data()), "r2d3c_transfers");
    std::vector<std::string> T, X;
    double x0 = 0.0, x1 = 0.0, x2 = 0.0;
    for (int k = 0; k < nb; ++k) {
      T.push_back(fortran_e(f0[k], 24, 15) + fortran_e(f1[k], 24, 15) + fortran_e(f2[k], 24, 15));
      x0 = f0[k] + x0;
      x1 = f1[k] + x1;
      x2 = f2[k] + x2;
      X.push_back(fortran_e(x0, 24, 15) + fortran_e(x1, 24, 15) + fortran_e(x2, 24, 15));
    }
    write_text(in.odir + "/transfer." + ext4 + ".txt", T);
    write_text(in.odir + "/fluxes." + ext4 + ".txt", X);
    append_line(dir + "/time_spec.txt", ext4 + fortran_f(time, 12, 6));
  }

  void fields() {  // :461-530
    if (++iu == 58) {
      iu = 48;
      ++id;
    }
    if (id == 58) {
      id = 48;
      ++ic;
    }
    const std::string ext = {(char)ic, (char)id, (char)iu};
    const char* names[4] = {"ps", "vz", "ww", "invlap_psi"};
    std::vector<double> r((size_t)n * n);
    for (int w = 0; w < 4; ++w) {
      check(r2d3c_get_field(ctx, w, r.data()), "r2d3c_get_field");
      write_field(in.odir + "/" + names[w] + "." + node + "." + ext + ".out", r);
    }
    append_line(dir + "/time_field.txt", ext + fortran_f(time, 12, 6));
  }

  double loop(long max_steps) {  // :393-615
    const r2d3c_params& p = in.p;
    long last = p.step;
    if (max_steps >= 0) last = std::min<long>(last, (long)ini + max_steps - 1);
    long t = ini;
    while (t <= last) {
      const bool dc = timec == p.cstep, ds = times == p.sstep, dt = timet == p.tstep;
      int k = 1;
      if (dc || ds || dt) {
        if (dc) {
          timec = 0;
          cond_check();
        }
        if (ds) {
          times = 0;
          spectra();
        }
        if (dt) {
          timet = 0;
          fields();
        }
      } else {
        // steps until the next output (the counters only grow between them)
        long gap = last - t + 1;
        const long g[3] = {(long)p.cstep - timec, (long)p.sstep - times, (long)p.tstep - timet};
        for (long x : g)
          if (x > 0) gap = std::min(gap, x);
        k = (int)std::max(1L, gap);
      }
      double dtl = 0.0;
      check(r2d3c_advance(ctx, k, R2D3C_DT_CFL, p.cfl, &time, &dtl, &seed, &seed1), "r2d3c_advance");
      timet += k;
      times += k;
      timec += k;
      t += k;
    }
    return time;
  }
};

}  // namespace

int main(int argc, char** argv) {
  int n = 0, precision = R2D3C_FP64;
  long max_steps = -1;
  std::string dir = ".";
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--n" && i + 1 < argc) n = std::atoi(argv[++i]);
    else if (a == "--dir" && i + 1 < argc) dir = argv[++i];
    else if (a == "--fp32") precision = R2D3C_FP32;
    else if (a == "--max-steps" && i + 1 < argc) max_steps = std::atol(argv[++i]);
    else {
      std::fprintf(stderr, "usage: %s --n N [--dir RUNDIR] [--fp32] [--max-steps K]\n", argv[0]);
      return 2;
    }
  }
  if (n <= 0) {
    std::fprintf(stderr, "--n N is required\n");
    return 2;
  }
  try {
    Run r(n, dir, precision);
    r.setup();
    const double t = r.loop(max_steps);
    std::printf("done: time = %.17g\n", t);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "rot2d3c_gpu: %s\n", e.what());
    return 1;
  }
  return 0;
}
