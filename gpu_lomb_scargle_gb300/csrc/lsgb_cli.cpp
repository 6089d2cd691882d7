// lsgb_cli.cpp -- lsgb_main, the reference's command-line front ends over this engine.
//
// Two syntaxes, as the reference's two programs have:
//   paper   (source/main.cu:92-252):
//       lsgb_main <data file> <min freq> <max freq> <num freqs> <mode 1|2|4|5> [options]
//   release (release/main.cu:179-398):
//       lsgb_main -f <data file> -min <f> -max <f> -fq <n> -m <mode 1|2|3|4> [options]
// Frequencies are angular. Modes: 1 GPU batch, 2 GPU one object, and the CPU modes
// (4/5 in the paper syntax, 3/4 in the release syntax).
// Options (both syntaxes; short and long forms):
//   -e, --error        generalized variant (id,t,mag,dmag rows); default: on when the file
//                      has 4 columns
//   -d, --double       double build (default: double for the paper syntax, float for the
//                      release syntax, as the reference programs default)
//   -nrp, --normpgram  normalize the standard periodogram by 2/(N var(y)); by default it is
//                      left unnormalized, as the reference's programs do (source/params.h:40
//                      NORMALIZEPGRAM 0, release/main.cu:376)
//   -n, --nthreads <k> CPU threads of the CPU modes (release/main.cu:330)
//   -ng, --ngpus <k>   accepted for the release syntax; this engine runs on one GPU
//   -ps, --printscreen             periods to stdout
//   -pf, --printfile <file>        periods to <file> (the paper's bestperiods.txt layout)
//   --top3 <file>                  three best periods and powers per object (the paper's
//                                  bestperiods_top_three.txt layout, PRINTPERIODS 3)
//   -ppf, --printpgramfile <file>  periodogram to <file> (the paper's pgram.txt layout)
//   -q, --quiet
// The data file is the reference's text format: comma-separated object id, time,
// magnitude[, dmag] per line (source/main.cu:1781-1843).
//
// The GPU modes call liblsgb.so (next to this executable) once: the three best frequencies
// of every object come out of the periodogram kernel itself (lsgb_periodogram_top3_host),
// and the periodogram is copied to the host only for -ppf. The double build computes in the
// plain FP64 form, the float build in the mixed form (LSGB_PRECISION=plain|mixed chooses).
// The CPU modes run the reference's CPU algorithm in the build's type (lsgb_cpu.h), and
// take the three best from the returned periodogram by the reference's three scans.
#include <dlfcn.h>
#include <limits.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <chrono>
#include <cmath>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/lsgb.h"
#include "lsgb_cpu.h"

namespace {

struct Args {
    std::string file, period_file, top3_file, pgram_file;
    double fmin = NAN, fmax = NAN;
    long nfreq = -1;
    int mode = 0;  // in the paper numbering (1, 2, 4, 5)
    int error = -1, dbl = -1;
    int nthreads = 0;  // 0: the OpenMP default
    bool print_screen = false, quiet = false, normalize = false;
};

[[noreturn]] void usage(const char *msg) {
    if (msg && *msg) fprintf(stderr, "lsgb_main: %s\n", msg);
    fprintf(stderr,
            "usage: lsgb_main <file> <min freq> <max freq> <num freqs> <mode 1|2|4|5> [options]\n"
            "       lsgb_main -f <file> -min <f> -max <f> -fq <n> -m <mode 1-4> [options]\n"
            "options: -e/--error -d/--double -nrp/--normpgram -n/--nthreads <k> -ng/--ngpus <k>\n"
            "         -ps/--printscreen -pf/--printfile <file> --top3 <file>\n"
            "         -ppf/--printpgramfile <file> -q/--quiet\n");
    exit(2);
}

bool is(const char *a, const char *s, const char *l) { return !strcmp(a, s) || !strcmp(a, l); }

double num(const char *s, const char *what) {
    char *end = nullptr;
    const double v = strtod(s, &end);
    if (end == s || *end) usage((std::string(what) + ": not a number: " + s).c_str());
    return v;
}

long inum(const char *s, const char *what) {
    char *end = nullptr;
    const long v = strtol(s, &end, 10);
    if (end == s || *end) usage((std::string(what) + ": not an integer: " + s).c_str());
    return v;
}

Args parse(int argc, char **argv) {
    Args a;
    bool release = false;
    std::vector<std::string> pos;
    for (int i = 1; i < argc; ++i) {
        const char *s = argv[i];
        auto val = [&](const char *what) -> const char * {
            if (i + 1 >= argc) usage((std::string(what) + " needs a value").c_str());
            return argv[++i];
        };
        if (is(s, "-h", "--help")) usage("");
        else if (is(s, "-f", "--filename")) { a.file = val(s); release = true; }
        else if (is(s, "-min", "--minfreq")) { a.fmin = num(val(s), "min freq"); release = true; }
        else if (is(s, "-max", "--maxfreq")) { a.fmax = num(val(s), "max freq"); release = true; }
        else if (is(s, "-fq", "--freq")) { a.nfreq = inum(val(s), "num freqs"); release = true; }
        else if (is(s, "-m", "--mode")) { a.mode = (int)inum(val(s), "mode"); release = true; }
        else if (is(s, "-e", "--error")) a.error = 1;
        else if (is(s, "-d", "--double")) a.dbl = 1;
        else if (is(s, "-ps", "--printscreen")) a.print_screen = true;
        else if (is(s, "-pf", "--printfile")) a.period_file = val(s);
        else if (!strcmp(s, "--top3")) a.top3_file = val(s);
        else if (is(s, "-ppf", "--printpgramfile")) a.pgram_file = val(s);
        else if (is(s, "-q", "--quiet")) a.quiet = true;
        else if (is(s, "-nrp", "--normpgram")) a.normalize = true;
        else if (is(s, "-n", "--nthreads")) {
            a.nthreads = (int)inum(val(s), "threads");
            if (a.nthreads < 1) usage("the number of threads must be positive");
        } else if (is(s, "-ng", "--ngpus")) {
            const long g = inum(val(s), "GPUs");
            if (g < 1) usage("the number of GPUs must be positive");
            if (g > 1) fprintf(stderr, "lsgb_main: one GPU is used (-ng %ld ignored)\n", g);
        }
        else if (s[0] == '-' && !(s[1] >= '0' && s[1] <= '9') && s[1] != '.') usage((std::string("unknown option ") + s).c_str());
        else pos.push_back(s);
    }
    if (!release) {
        if (pos.size() != 5) usage("expected <file> <min freq> <max freq> <num freqs> <mode>");
        a.file = pos[0];
        a.fmin = num(pos[1].c_str(), "min freq");
        a.fmax = num(pos[2].c_str(), "max freq");
        a.nfreq = inum(pos[3].c_str(), "num freqs");
        a.mode = (int)inum(pos[4].c_str(), "mode");
        if (a.dbl < 0) a.dbl = 1;
    } else {
        if (!pos.empty()) usage("positional arguments mixed with -f/-min/-max/-fq/-m");
        if (a.mode == 3) a.mode = 4;       // release numbering -> paper numbering
        else if (a.mode == 4) a.mode = 5;
        if (a.dbl < 0) a.dbl = 0;
    }
    if (a.file.empty()) usage("a data file is required");
    if (!std::isfinite(a.fmin) || !std::isfinite(a.fmax)) usage("min and max frequency are required");
    if (a.nfreq <= 0 || a.nfreq > 0xffffffffL) usage("the number of frequencies must be positive");
    if (a.mode != 1 && a.mode != 2 && a.mode != 4 && a.mode != 5) usage("unknown mode");
    return a;
}

struct Data {
    std::vector<uint32_t> id;
    std::vector<double> t, y, dy;
    int columns = 0;
};

Data read_file(const std::string &path) {
    std::ifstream in(path);
    if (!in) {
        fprintf(stderr, "lsgb_main: cannot open %s\n", path.c_str());
        exit(1);
    }
    Data d;
    std::string line;
    size_t lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        double v[4];
        int k = 0;
        const char *p = line.c_str();
        while (*p && k < 4) {
            while (*p == ' ' || *p == '\t' || *p == ',') ++p;
            if (!*p || *p == '\r') break;
            char *end = nullptr;
            v[k] = strtod(p, &end);
            if (end == p) break;
            ++k;
            p = end;
        }
        if (k == 0) continue;
        if (k < 3) {
            fprintf(stderr, "lsgb_main: %s:%zu: expected id, time, mag[, dmag]\n", path.c_str(), lineno);
            exit(1);
        }
        if (!d.columns) d.columns = k;
        d.id.push_back((uint32_t)v[0]);
        d.t.push_back(v[1]);
        d.y.push_back(v[2]);
        d.dy.push_back(k >= 4 ? v[3] : 1.0);
    }
    return d;
}

std::string exe_dir() {
    char buf[PATH_MAX];
    ssize_t n = readlink("/proc/self/exe", buf, sizeof(buf) - 1);
    if (n <= 0) return ".";
    buf[n] = 0;
    std::string s(buf);
    return s.substr(0, s.find_last_of('/'));
}

// The reference's three scans over one periodogram (source/main.cu:1165-1219): the three
// largest positive powers at distinct indices, best first, the first index among equal
// powers; (0, index 0) where there are fewer.
template <typename T>
void top3_scan(const T *p, size_t nf, uint32_t idx[3], T pw[3]) {
    for (int r = 0; r < 3; ++r) {
        idx[r] = 0;
        pw[r] = 0;
        for (size_t k = 0; k < nf; ++k) {
            const bool taken = (r >= 1 && k == idx[0]) || (r >= 2 && k == idx[1]);
            if (!taken && pw[r] < p[k]) {
                pw[r] = p[k];
                idx[r] = (uint32_t)k;
            }
        }
    }
}

typedef int (*EngineCreateFn)(int, lsgb_engine **);
typedef const char *(*LastErrorFn)(void);
typedef int (*Top3HostFn)(lsgb_engine *, int, int, int, const void *, const void *, const void *,
                          const uint64_t *, uint32_t, double, double, uint32_t, int, void *,
                          uint32_t *, void *);

template <typename T>
int run(const Args &a, Data &d) {
    const bool err = a.error == 1, gpu = a.mode == 1 || a.mode == 2;
    const size_t rows = d.t.size();
    std::vector<T> t(d.t.begin(), d.t.end()), y(d.y.begin(), d.y.end()), dy(d.dy.begin(), d.dy.end());
    // objects: runs of equal ids (source/main.cu:468-510); one object in the single modes
    std::vector<uint64_t> offs{0};
    if (a.mode == 1 || a.mode == 4)
        for (size_t i = 1; i < rows; ++i)
            if (d.id[i] != d.id[i - 1]) offs.push_back(i);
    offs.push_back(rows);
    const uint32_t nobj = (uint32_t)offs.size() - 1;
    const size_t nf = (size_t)a.nfreq;
    // The reference's drivers take the limits in the build's type (source/main.cu:742, :1358).
    const T fminT = (T)a.fmin, fmaxT = (T)a.fmax;
    printf("\nDataset file: %s", a.file.c_str());
    printf("\nMinimum Frequency: %f", a.fmin);
    printf("\nMaximum Frequency: %f", a.fmax);
    printf("\nNumber of frequencies to test: %zu", nf);
    printf("\nMode: %d", a.mode);
    if (err) printf("\nExecuting L-S variant from AstroPy that propogates error and floats the mean");
    printf("\nData import: Total rows: %zu", rows);
    if (a.mode == 1 || a.mode == 4) printf("\nUnique objects in file: %u", nobj);
    const bool want_pgram = !a.pgram_file.empty();
    std::vector<T> pgram;
    std::vector<uint32_t> idx3(3 * (size_t)nobj);
    std::vector<T> pow3(3 * (size_t)nobj);
    double step_period = 0;  // GPU modes: the frequency step of the period formula
    T step_cpu = 0;          // CPU modes: the step in the build's type
    const auto t0 = std::chrono::steady_clock::now();
    if (gpu) {
        const std::string lib = exe_dir() + "/liblsgb.so";
        void *h = dlopen(lib.c_str(), RTLD_NOW | RTLD_LOCAL);
        if (!h) {
            fprintf(stderr, "lsgb_main: %s\n", dlerror());
            return 1;
        }
        auto create = (EngineCreateFn)dlsym(h, "lsgb_engine_create");
        auto last_error = (LastErrorFn)dlsym(h, "lsgb_last_error");
        auto top3 = (Top3HostFn)dlsym(h, "lsgb_periodogram_top3_host");
        if (!create || !last_error || !top3) {
            fprintf(stderr, "lsgb_main: %s lacks the lsgb_* entry points\n", lib.c_str());
            return 1;
        }
        // the generalized variant centers y per object first (source/main.cu:1045, :187)
        if (err)
            for (uint32_t o = 0; o < nobj; ++o)
                lsgb_cpu::precenter<T>(y.data() + offs[o], dy.data() + offs[o],
                                       (uint32_t)(offs[o + 1] - offs[o]));
        int precision = a.dbl ? LSGB_PLAIN_FP64 : LSGB_MIXED;
        const char *pe = getenv("LSGB_PRECISION");
        if (pe && !strcmp(pe, "plain")) precision = LSGB_PLAIN_FP64;
        if (pe && !strcmp(pe, "mixed")) precision = LSGB_MIXED;
        // the kernels' grid: fmin + k * df, df computed in double and held in the build's
        // type (source/kernel.cu:517)
        const double fmin = (double)fminT;
        const double df = (double)(T)(((double)fmaxT - (double)fminT) / (nf * 1.0));
        lsgb_engine *eng = nullptr;
        int rc = create(0, &eng);
        if (rc == LSGB_OK) {
            if (want_pgram) pgram.assign((size_t)nobj * nf, T(0));
            const auto tk = std::chrono::steady_clock::now();
            rc = top3(eng, err ? LSGB_GENERALIZED : LSGB_STANDARD, precision,
                      sizeof(T) == 4 ? LSGB_F32 : LSGB_F64, t.data(), y.data(),
                      err ? dy.data() : nullptr, offs.data(), nobj, fmin, df, (uint32_t)nf,
                      (!err && a.normalize) ? 1 : 0, want_pgram ? pgram.data() : nullptr,
                      idx3.data(), pow3.data());
            printf("\nTime to compute kernel: %f",
                   std::chrono::duration<double>(std::chrono::steady_clock::now() - tk).count());
        }
        if (rc != LSGB_OK) {
            fprintf(stderr, "lsgb_main: GPU computation failed: %s\n", last_error());
            return 1;
        }
        // the period formula of the GPU drivers uses the step in double (source/main.cu:1140)
        step_period = ((double)fmaxT - (double)fminT) / (nf * 1.0);
    } else {
#ifdef _OPENMP
        if (a.nthreads > 0) omp_set_num_threads(a.nthreads);
#endif
        pgram.assign((size_t)nobj * nf, T(0));
        const T freqStep = (fmaxT - fminT) / (nf * 1.0);
        // objects in parallel (MODE 4), or frequencies in parallel within one (MODE 5), as
        // the reference's CPU modes (source/main.cu:1487, :1617)
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) if (a.mode == 4)
#endif
        for (uint32_t o = 0; o < nobj; ++o) {
            const uint64_t r0 = offs[o];
            const uint32_t n = (uint32_t)(offs[o + 1] - r0);
            T *pg = pgram.data() + (size_t)o * nf;
            if (err)
                lsgb_cpu::object_pgram<T, 1>(t.data() + r0, y.data() + r0, dy.data() + r0, n,
                                             (uint32_t)nf, fminT, freqStep, pg, a.mode == 5, false);
            else
                lsgb_cpu::object_pgram<T, 0>(t.data() + r0, y.data() + r0, dy.data() + r0, n,
                                             (uint32_t)nf, fminT, freqStep, pg, a.mode == 5,
                                             a.normalize);
            top3_scan(pg, nf, idx3.data() + 3 * (size_t)o, pow3.data() + 3 * (size_t)o);
        }
        step_cpu = freqStep;
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // period = 2 pi / omega: in double from the double step in the GPU drivers
    // (source/main.cu:1140-1160), in the build's type in the CPU modes (computePeriod,
    // source/main.cu:1545-1563)
    std::vector<double> per(3 * (size_t)nobj);
    double sum = 0;
    for (size_t i = 0; i < per.size(); ++i)
        per[i] = gpu ? (1.0 / ((double)fminT + (idx3[i] * step_period))) * 2.0 * M_PI
                     : (double)(T)((1.0 / (fminT + (idx3[i] * step_cpu))) * 2.0 * M_PI);
    for (uint32_t o = 0; o < nobj; ++o) sum += per[3 * (size_t)o];
    const uint32_t single_id = d.id.empty() ? 0 : d.id[0];
    auto obj_id = [&](uint32_t o) { return (a.mode == 2 || a.mode == 5) ? single_id : d.id[offs[o]]; };
    if (a.mode == 2) {
        printf("\nPeriod: %f", per[0]);
        printf("\nMaximum power at found period: %f", (double)pow3[0]);
    }
    if (!a.quiet) printf("\nTotal time to compute batch: %f", secs);
    if (a.mode == 1 || a.mode == 4)
        printf("\n[Validation] Sum of all periods: %f\n", sum);
    else
        printf("\n[Validation] Period: %f, Power: %f\n", per[0], (double)pow3[0]);
    if (a.print_screen)
        for (uint32_t o = 0; o < nobj; ++o)
            printf("Object: %u Period: %f, Power: %f \n", obj_id(o), per[3 * (size_t)o],
                   (double)pow3[3 * (size_t)o]);
    if (!a.period_file.empty()) {
        std::ofstream f(a.period_file);
        f.precision(6);
        for (uint32_t o = 0; o < nobj; ++o)
            f << obj_id(o) << ", " << per[3 * (size_t)o] << ", " << pow3[3 * (size_t)o] << "\n";
    }
    if (!a.top3_file.empty()) {
        std::ofstream f(a.top3_file);
        f.precision(6);
        for (uint32_t o = 0; o < nobj; ++o) {
            const size_t b = 3 * (size_t)o;
            f << obj_id(o) << ", " << per[b] << ", " << per[b + 1] << ", " << per[b + 2] << ", "
              << pow3[b] << ", " << pow3[b + 1] << ", " << pow3[b + 2] << "\n";
        }
    }
    if (want_pgram) {
        std::ofstream f(a.pgram_file);
        f.precision(4);
        for (uint32_t o = 0; o < nobj; ++o) {
            f << obj_id(o) << ", ";
            for (size_t k = 0; k < nf; ++k) f << pgram[(size_t)o * nf + k] << ", ";
            f << "\n";
        }
    }
    // the reference appends a line per run to gpu_stats.txt in the working directory
    const char *no = getenv("LSGB_NO_STATS");
    if (!(no && !strcmp(no, "1"))) {
        std::ofstream g("gpu_stats.txt", std::ios::app);
        g << secs << ", " << a.file << ", Sum of periods: " << sum << ", Min/Max Freq: " << a.fmin
          << "/" << a.fmax << ",  Num tested freq: " << nf << ", MODE: " << a.mode
          << ", ERROR/DTYPE/ENGINE: " << (err ? 1 : 0) << ", " << (sizeof(T) == 4 ? "float" : "double")
          << ", lsgb" << std::endl;
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    Args a = parse(argc, argv);
    Data d = read_file(a.file);
    if (d.t.empty()) {
        fprintf(stderr, "lsgb_main: %s has no observations\n", a.file.c_str());
        return 1;
    }
    if (a.error < 0) a.error = d.columns >= 4 ? 1 : 0;
    if (a.error == 1 && d.columns < 4) {
        fprintf(stderr, "lsgb_main: the generalized variant needs a dmag column\n");
        return 1;
    }
    return a.dbl ? run<double>(a, d) : run<float>(a, d);
}
