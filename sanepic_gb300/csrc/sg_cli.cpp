// sg_cli.cpp -- `sanepic`, the drop-in executable for the reference's
// map-making run (patanch/SANEPIC src/sanepic.cc main, invoked by
// scripts/run_sanepic.sh) on one GPU through libsanepic_gpu's C ABI.
//
// Same command line (the getopt string of sanepic.cc:315-317), same input
// files and the same output files and names.  No mpirun is needed: one
// process drives one GPU.  What differs on purpose:
//  * errors print a message and exit(1) instead of undefined behaviour
//    (missing or short input files, segment lists that do not match -l/-n);
//  * options of code paths that are not part of the map-maker's hot path
//    (-o dipole, -c leakage recalibration, -b galactic leakage) are refused
//    when switched on; -E 1 stops like the reference ("NOT IMPLEMENTED YET");
//    the other options are accepted and ignored, as the reference ignores them;
//  * -r (with -R: one gain per detector) runs the reference's outer loop of
//    map-making and gain fits (sanepic.cc:1041-1042, 2123-2316) with its fit
//    corrected (sg_fit_gains: the reference's fits carry a factor 4 and its
//    loop diverges); the orbital-dipole timelines orbdip_<detector> it reads
//    must be absent or zero (the -o path is not implemented);
//  * SANEPIC_GPU_PRECISION (f64 | f32), SANEPIC_GPU_PRECOND (diag | bj3),
//    SANEPIC_GPU_DEVICE and SANEPIC_GPU_STOP select what the reference fixes:
//    FP64 and its diagonal preconditioner by default, stop at 1e-15;
//    SANEPIC_GPU_POL_RCOND > 0 also masks Q/U of pixels whose 3 x 3 hit block
//    is that ill-conditioned (sg_set_pol_rcond; default 0, the reference's rule).
#include <getopt.h>

#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "sanepic_gpu.h"

namespace {

// sanepic.cc:315-317
const char* const kOptions =
    "F:Z:f:n:l:d:D:C:H:h:w:J:o:O:B:R:X:G:P:e:p:A:m:k:K:u:c:N:n:L:g:r:M:E:j:z:b:I:i:";

[[noreturn]] void die(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  fputc('\n', stderr);
  exit(1);
}

void usage(const char* prog) {
  fprintf(stderr,
          "usage: %s -F <tod dir> -B <tod suffix> -Z <pointing prefix> -f <segment list>\n"
          "          -n <segments> -l <samples per segment> -d <detectors>\n"
          "          (-C <detector> ... | -D <detector list file>) -X <bolometer_info>\n"
          "          -k <iSpf prefix> -u <iSpf length> -N <nside> -p 1 -O <output prefix>\n"
          "          -e <output id> [-h <hwp> -w <hwp rad/sample>] [-I <start map>]\n"
          "          [-i <write iteration maps> -j <every>] [-P <pointing suffix>]\n"
          "          [-r 1 [-R 1]]  gain recalibration loop (per tile; -R: per detector)\n"
          "environment: SANEPIC_GPU_PRECISION=f64|f32  SANEPIC_GPU_PRECOND=diag|bj3\n"
          "             SANEPIC_GPU_DEVICE=<ordinal>   SANEPIC_GPU_STOP=<crit>\n"
          "             SANEPIC_GPU_POL_RCOND=<min reciprocal condition of a pixel's Q/U>\n",
          prog);
}

struct Args {
  std::string dirfile, dirfilep, segfile, outdir, bext, pext, termin, noise_prefix, detinfo,
      init_map;
  bool have_pointing_dir = false, have_init = false;
  long ndet = 0, nseg = 0, ns = 0, nssp = 0, nside = 0;
  int pol = 0, hwp = 0, iterw = 10, write_iter = 1;
  bool recalib = false, recal_global = false;  // -r, -R (sanepic.cc:364, 388)
  double omega = 0.0;
  std::vector<std::string> bolos;
};

// first word of every non-empty, non-comment line (read_bolofile, sanepic.cc:3134-3157)
void read_bolo_list(const std::string& fname, std::vector<std::string>& out) {
  std::ifstream in(fname);
  if (!in.is_open()) die("Error opening bolometer file '%s'. Exiting.", fname.c_str());
  std::string line;
  while (std::getline(in, line)) {
    const size_t b = line.find_first_not_of(" \t\r");
    if (b == std::string::npos || line[b] == '#') continue;
    const size_t e = line.find_first_of(" \t\r", b);
    out.push_back(line.substr(b, e == std::string::npos ? std::string::npos : e - b));
  }
}

// rows "num pnum lel xel angle TEL NAME"; the last row naming `bolo` wins
// (read_bolo_offsets, sanepic.cc:3159-3185).  Returns {xel, lel, angle}.
void read_bolo_offsets(const std::string& bolo, const std::string& file, double* off) {
  FILE* fp = fopen(file.c_str(), "r");
  if (!fp) die("ERROR: Can't find offset file. Exiting. ");
  long num, pnum;
  double lel, xel, angl;
  char tel[300], name[300];
  bool found = false;
  while (fscanf(fp, "%ld%ld%lf%lf%lf%299s%299s", &num, &pnum, &lel, &xel, &angl, tel, name) == 7) {
    if (bolo == name) {
      found = true;
      off[0] = xel;
      off[1] = lel;
      off[2] = angl;
    }
  }
  fclose(fp);
  if (!found) die("Bolometer name not found in offset list");
}

// n native-endian values starting at element `first` (ReadDoubleVECT /
// ReadLongVECT, sanepic.cc:3083-3132), with the size checks the reference lacks
template <typename T>
void read_vector(const std::string& path, long first, long n, std::vector<T>& out) {
  FILE* fp = fopen(path.c_str(), "rb");
  if (!fp) die("cannot open %s: %s", path.c_str(), strerror(errno));
  out.resize(n);
  if (fseek(fp, first * (long)sizeof(T), SEEK_SET) != 0)
    die("cannot seek to element %ld of %s", first, path.c_str());
  const size_t got = fread(out.data(), sizeof(T), n, fp);
  fclose(fp);
  if ((long)got != n)
    die("%s: expected %ld values from element %ld, found %zu", path.c_str(), n, first, got);
}

void write_vector(const std::string& path, const double* v, long n) {
  FILE* fp = fopen(path.c_str(), "wb");
  if (!fp) die("cannot write %s: %s", path.c_str(), strerror(errno));
  const size_t put = fwrite(v, sizeof(double), n, fp);
  fclose(fp);
  if ((long)put != n) printf("WARNING, PROBLEM WITH WRITTEN DATA\n");
}

long parse_long(const char* s, char opt) {
  char* end = nullptr;
  const long v = strtol(s, &end, 10);
  if (end == s) die("option -%c: '%s' is not an integer", opt, s);
  return v;
}

Args parse(int argc, char** argv) {
  Args a;
  int c;
  while ((c = getopt(argc, argv, kOptions)) != -1) {
    switch (c) {
      case 'F': a.dirfile = optarg; break;
      case 'Z': a.dirfilep = optarg; a.have_pointing_dir = true; break;
      case 'f': a.segfile = optarg; break;
      case 'p': a.pol = (int)parse_long(optarg, 'p'); break;
      case 'd': a.ndet = parse_long(optarg, 'd'); break;
      case 'D': {
        read_bolo_list(optarg, a.bolos);
        fprintf(stderr, "num bolos: %zu\n", a.bolos.size());
        break;
      }
      case 'C': a.bolos.push_back(optarg); break;
      case 'O': a.outdir = optarg; break;
      case 'B': a.bext = optarg; break;
      case 'X': a.detinfo = optarg; break;
      case 'P': a.pext = optarg; break;
      case 'e': a.termin = optarg; break;
      case 'k': a.noise_prefix = optarg; break;
      case 'u': a.nssp = parse_long(optarg, 'u'); break;
      case 'N': a.nside = parse_long(optarg, 'N'); break;
      case 'n': a.nseg = parse_long(optarg, 'n'); break;
      case 'l': a.ns = parse_long(optarg, 'l'); break;
      case 'j': a.iterw = (int)parse_long(optarg, 'j'); break;
      case 'h': a.hwp = atoi(optarg) != 0; break;
      case 'w': a.omega = atof(optarg); break;
      case 'I': a.init_map = optarg; a.have_init = true; break;
      case 'i': a.write_iter = atoi(optarg) != 0; break;
      case 'E':
        if (atoi(optarg)) {  // correlated noise (sanepic.cc:515-517)
          printf("NOT IMPLEMENTED YET\n");
          exit(0);
        }
        break;
      case 'r': a.recalib = atoi(optarg) != 0; break;
      case 'R': a.recal_global = atoi(optarg) != 0; break;
      case 'o': case 'c': case 'b':
        if (atoi(optarg))
          die("option -%c %s selects a path this executable does not implement "
              "(dipole / leakage recalibration / galactic leakage)", c, optarg);
        break;
      case 'H': case 'J': case 'G': case 'A': case 'm': case 'K': case 'L': case 'g':
      case 'M': case 'z':
        break;  // parsed and unused on the map-making path
      default:
        fprintf(stderr, "Option '%c' not valid. Exiting.\n\n", (char)optopt);
        usage(argv[0]);
        exit(1);
    }
  }
  if (!a.have_pointing_dir) a.dirfilep = a.dirfile;
  return a;
}

int env_int(const char* name, int dflt) {
  const char* v = getenv(name);
  return v && *v ? atoi(v) : dflt;
}

}  // namespace

namespace {

struct Run {
  const Args* a;
  sg_ctx* ctx;
  long npixfull;
  std::vector<double> full;
  int rloop = 1;  // the outer loop of -r (sanepic.cc:1041)

  void check(int rc, const char* what) {
    if (rc != SG_OK) die("%s failed (%d): %s", what, rc, sg_last_error(ctx));
  }
  void write_map(int kind, const std::string& name) {
    check(sg_get_map(ctx, kind, full.data()), "sg_get_map");
    write_vector(name, full.data(), npixfull);
  }
};

// per-iteration output: the reference's line (sanepic.cc:1607-1609), the
// noise/hit maps at iteration 1 (sanepic.cc:1616-1707) and, with -i, the
// running maps every -j iterations (sanepic.cc:1709-1745)
int on_iteration(void* user, int iter, double crit, double crit2, double chi2) {
  Run* r = static_cast<Run*>(user);
  const Args& a = *r->a;
  printf("iter = %d, crit = %10.15g, crit2 = %10.15g, chi2 = %10.15g\n", iter, crit, crit2, chi2);
  fflush(stdout);
  const std::string& O = a.outdir;
  const std::string& e = a.termin;
  if (r->rloop != 1) return 0;  // the maps below only in the first loop (sanepic.cc:1616, 1711)
  if (iter == 1) {
    r->write_map(SG_MAP_NVAR, O + "_NVAR" + e);
    r->write_map(SG_MAP_HITS, O + "_HITS" + e);
    r->write_map(SG_MAP_COS2P, O + "_COS2P_" + e);
    r->write_map(SG_MAP_SIN2P, O + "_SIN2P_" + e);
    r->write_map(SG_MAP_Q_NVAR, O + "_Q_NVAR" + e);
    r->write_map(SG_MAP_U_NVAR, O + "_U_NVAR" + e);
    r->write_map(SG_MAP_POL_HITS, O + "_POL_HITS" + e);
  }
  if (a.iterw && iter % a.iterw == 0 && a.write_iter) {
    const std::string s = "_" + std::to_string(iter);
    r->write_map(SG_MAP_I, O + "_I" + e + s);
    r->write_map(SG_MAP_Q, O + "_Q" + e + s);
    r->write_map(SG_MAP_U, O + "_U" + e + s);
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  const Args a = parse(argc, argv);
  if (a.ndet <= 0) die("-d: the number of detectors must be positive");
  if (a.nseg <= 0) die("-n: the number of segments must be positive");
  if (a.ns <= 0) die("-l: the segment length must be positive");
  if (a.nssp <= 0) die("-u: the iSpf length must be positive");
  if (a.nside <= 0) die("-N: nside must be positive");
  if (a.pol != 1) die("-p %d: only pol=1 is supported (the reference's pol=0 path is broken)", a.pol);
  if ((long)a.bolos.size() < a.ndet)
    die("-d %ld detectors but only %zu names given (-C / -D)", a.ndet, a.bolos.size());

  // detector offsets and angles (sanepic.cc:452-464)
  const double d2r = M_PI / 180.0;
  std::vector<sg_det> dets(a.ndet);
  for (long i = 0; i < a.ndet; i++) {
    double off[3];
    read_bolo_offsets(a.bolos[i], a.detinfo, off);
    dets[i].offx = off[1] * d2r;
    dets[i].offy = off[0] * d2r;
    dets[i].psi = off[2] * d2r;
    printf("Angle detector %ld = %10.15g\n", i, dets[i].psi);
  }
  printf("nsegtot = %ld\n", a.nseg);

  // segment list (sanepic.cc:496-501, 668-672)
  std::vector<long> seg;
  read_vector(a.segfile, 0, 2 * a.nseg, seg);
  std::vector<long> isampmin(a.nseg);
  long nsamp_total = 0;
  for (long i = 0; i < a.nseg; i++) {
    const long lo = seg[2 * i], hi = seg[2 * i + 1];
    if (hi - lo + 1 != a.ns) {
      printf("Problem with segment size: %ld, %ld\n", hi - lo, a.ns);
      exit(1);
    }
    if (lo < 0) die("segment %ld starts at negative sample %ld", i, lo);
    isampmin[i] = lo;
    if (hi + 1 > nsamp_total) nsamp_total = hi + 1;
  }

  // boresight pointing, full timeline (sanepic.cc:680-692)
  std::vector<double> ra, dec, psi;
  read_vector(a.dirfilep + "ra" + a.pext + ".bi", 0, nsamp_total, ra);
  read_vector(a.dirfilep + "dec" + a.pext + ".bi", 0, nsamp_total, dec);
  read_vector(a.dirfilep + "psi" + a.pext + ".bi", 0, nsamp_total, psi);

  const char* prec = getenv("SANEPIC_GPU_PRECISION");
  const char* pc = getenv("SANEPIC_GPU_PRECOND");
  const char* stop = getenv("SANEPIC_GPU_STOP");
  sg_desc desc{};
  desc.ns = a.ns;
  desc.nseg = a.nseg;
  desc.ndet = a.ndet;
  desc.nside = a.nside;
  desc.pol = a.pol;
  desc.hwp = a.hwp;
  desc.omega = a.omega;
  desc.precision = (prec && strcmp(prec, "f32") == 0) ? SG_F32 : SG_F64;
  desc.device = env_int("SANEPIC_GPU_DEVICE", 0);
  if (prec && strcmp(prec, "f32") != 0 && strcmp(prec, "f64") != 0)
    die("SANEPIC_GPU_PRECISION must be f64 or f32");
  if (pc && strcmp(pc, "diag") != 0 && strcmp(pc, "bj3") != 0)
    die("SANEPIC_GPU_PRECOND must be diag or bj3");

  Run run{&a, nullptr, 12 * a.nside * a.nside, {}};
  run.full.resize(run.npixfull);
  const int rc0 = sg_create(&run.ctx, &desc);
  if (rc0 != SG_OK) die("sg_create failed (%d): %s", rc0, run.ctx ? sg_last_error(run.ctx) : "");
  run.check(sg_set_pointing(run.ctx, ra.data(), dec.data(), psi.data(), nsamp_total,
                            isampmin.data(), dets.data()),
            "sg_set_pointing");
  if (const char* rc = getenv("SANEPIC_GPU_POL_RCOND")) {
    char* end = nullptr;
    const double v = strtod(rc, &end);
    if (end == rc || *end != '\0') die("SANEPIC_GPU_POL_RCOND must be a number");
    run.check(sg_set_pol_rcond(run.ctx, v), "sg_set_pol_rcond");
  }
  ra = std::vector<double>();
  dec = std::vector<double>();
  psi = std::vector<double>();

  // noise spectra (sanepic.cc:519-539) and TODs (sanepic.cc:776-790)
  std::vector<double> buf;
  for (long i = 0; i < a.ndet; i++) {
    const std::string nf = a.noise_prefix + a.bolos[i];
    printf("NoiseSpFiledet = %s\n", nf.c_str());
    read_vector(nf, 0, a.nssp, buf);
    run.check(sg_set_noise(run.ctx, i, buf.data(), a.nssp), "sg_set_noise");
  }
  for (long i = 0; i < a.ndet; i++) {
    const std::string tf = a.dirfile + "/data_" + a.bolos[i] + a.bext + ".bi";
    read_vector(tf, 0, nsamp_total, buf);
    for (long s = 0; s < nsamp_total; s++)
      if (std::isnan(buf[s])) printf("NAN DETECTED IN %s, data[%ld] = %10.15g\n", tf.c_str(), s, buf[s]);
    run.check(sg_set_tod(run.ctx, i, buf.data(), nsamp_total), "sg_set_tod");
  }

  // -r reads the orbital dipole of every detector (sanepic.cc:702-712): this
  // executable takes it as zero, so a file that holds anything else is refused
  if (a.recalib) {
    for (long i = 0; i < a.ndet; i++) {
      const std::string df = a.dirfile + "/orbdip_" + a.bolos[i];
      FILE* fp = fopen(df.c_str(), "rb");
      if (!fp) continue;
      fclose(fp);
      read_vector(df, 0, nsamp_total, buf);
      for (long g = 0; g < a.nseg; g++)
        for (long s = isampmin[g]; s < isampmin[g] + a.ns; s++)
          if (buf[s] != 0.0)
            die("%s: nonzero orbital dipole (the -o path is not implemented)", df.c_str());
    }
  }

  double chi20 = 0.0;
  run.check(sg_rhs(run.ctx, &chi20), "sg_rhs");
  printf("PtNd Computed...\n");
  const long npix = sg_npix(run.ctx);
  std::vector<double> x0;
  if (a.have_init) read_vector(a.init_map, 0, 3 * npix, x0);  // sanepic.cc:1209-1214

  sg_solve_opts o{};
  o.precond = (pc && strcmp(pc, "bj3") == 0) ? SG_PRECOND_BJ3 : SG_PRECOND_DIAG;
  o.stop_crit = stop && *stop ? atof(stop) : 1e-15;  // sanepic.cc:1037
  o.maxiter = 2000;                                  // sanepic.cc:1415
  o.refresh_every = 10;
  o.x0 = a.have_init ? x0.data() : nullptr;
  o.use_graph = 1;
  o.on_iteration = on_iteration;
  o.user = &run;
  sg_report rep{};
  run.check(sg_solve(run.ctx, &o, &rep), "sg_solve");
  printf("\n");

  // final maps of each loop (sanepic.cc:1770-1801)
  const std::string& O = a.outdir;
  std::vector<double> sol(3 * npix);
  auto write_loop_maps = [&]() {
    const std::string tail = "_" + a.termin + "_" + std::to_string(run.rloop);
    run.check(sg_get_solution(run.ctx, sol.data()), "sg_get_solution");
    write_vector(O + "_A" + tail, sol.data(), 3 * npix);
    run.write_map(SG_MAP_I, O + "_I" + tail);
    run.write_map(SG_MAP_Q, O + "_Q" + tail);
    run.write_map(SG_MAP_U, O + "_U" + tail);
  };
  write_loop_maps();
  int total_iters = rep.iterations;

  if (a.recalib) {
    // the outer loop (sanepic.cc:1041-1042, 2123-2316): fit the gains to the
    // map, write them (relCalib.dat<loop>, in the working directory as the
    // reference does), and make the map again from the previous one with the
    // new gains, until a loop starts already converged (its var0 / var00 at
    // most the stop criterion) or the 500th loop
    const double stop_crit = o.stop_crit;
    const double var00_1 = rep.var00;
    double var0_ratio = rep.crit0;  // var0 / var00 of the loop just made
    std::vector<double> gains(a.ndet * a.nseg, 1.0);
    while (true) {
      double x2b = 0.0, x2a = 0.0;
      run.check(sg_fit_gains(run.ctx, a.recal_global ? 1 : 0, gains.data(), &x2b, &x2a),
                "sg_fit_gains");
      printf("Before recal chi2 = %10.15g\n", x2b);
      if (a.recal_global)
        for (long d = 0; d < a.ndet; d++) printf("Coef calib det %ld is %10.15g\n", d, gains[d]);
      printf("After recal chi2 = %10.15g\n", x2a);
      fflush(stdout);
      write_vector("relCalib.dat" + std::to_string(run.rloop), gains.data(), a.ndet * a.nseg);
      run.rloop += 1;
      if (!(run.rloop < 500 && var0_ratio > stop_crit)) break;
      run.check(sg_set_gains(run.ctx, gains.data()), "sg_set_gains");
      run.check(sg_rhs(run.ctx, nullptr), "sg_rhs");
      o.x0 = sol.data();  // the previous loop's map (sanepic.cc:1226-1232)
      run.check(sg_solve(run.ctx, &o, &rep), "sg_solve");
      printf("\n");
      var0_ratio = rep.crit0 * rep.var00 / var00_1;
      total_iters += rep.iterations;
      write_loop_maps();
    }
  }
  fprintf(stderr, "sanepic (GPU): %d loop(s), %d iterations, crit %.3e, %.3f s last solve (%.1f it/s)\n",
          a.recalib ? run.rloop - 1 : 1, total_iters, rep.crit, rep.solve_seconds,
          rep.iter_per_sec);
  sg_destroy(run.ctx);
  return 0;
}
