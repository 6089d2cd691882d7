// lsgb_cli.cpp -- lsgb_main, the reference's command-line front ends over the drop-in
// libraries.
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
//   -ps, --printscreen             periods to stdout
//   -pf, --printfile <file>        periods to <file> (the paper's bestperiods.txt layout)
//   --top3 <file>                  top three periods/powers per object (bestperiods_top_three.txt)
//   -ppf, --printpgramfile <file>  periodogram to <file> (the paper's pgram.txt layout)
//   -q, --quiet
// The data file is the reference's text format: comma-separated object id, time,
// magnitude[, dmag] per line (source/main.cu:1781-1843). The work is done by
// LombScarglePy of the matching libpyls*.so next to this executable, so the results
// are those of the drop-in libraries; its stdout lines and gpu_stats.txt append are
// the reference's.
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

namespace {

struct Args {
    std::string file, period_file, top3_file, pgram_file;
    double fmin = NAN, fmax = NAN;
    long nfreq = -1;
    int mode = 0;  // in the paper numbering (1, 2, 4, 5)
    int error = -1, dbl = -1;
    bool print_screen = false, quiet = false;
};

[[noreturn]] void usage(const char *msg) {
    if (msg && *msg) fprintf(stderr, "lsgb_main: %s\n", msg);
    fprintf(stderr,
            "usage: lsgb_main <file> <min freq> <max freq> <num freqs> <mode 1|2|4|5> [options]\n"
            "       lsgb_main -f <file> -min <f> -max <f> -fq <n> -m <mode 1-4> [options]\n"
            "options: -e/--error -d/--double -ps/--printscreen -pf/--printfile <file>\n"
            "         --top3 <file> -ppf/--printpgramfile <file> -q/--quiet\n");
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

template <typename T>
int run(const Args &a, Data &d) {
    const bool err = a.error == 1;
    const std::string lib = exe_dir() + "/libpyls" + (err ? "error" : "noerror") +
                            (sizeof(T) == 4 ? "float" : "double") + ".so";
    void *h = dlopen(lib.c_str(), RTLD_NOW | RTLD_LOCAL);
    if (!h) {
        fprintf(stderr, "lsgb_main: %s\n", dlerror());
        return 1;
    }
    typedef void (*Fn)(unsigned *, T *, T *, T *, unsigned, double, double, unsigned, int, T *);
    typedef int (*StatusFn)();
    Fn fn = (Fn)dlsym(h, "LombScarglePy");
    StatusFn st = (StatusFn)dlsym(h, "LombScarglePy_last_status");
    if (!fn || !st) {
        fprintf(stderr, "lsgb_main: %s does not export LombScarglePy\n", lib.c_str());
        return 1;
    }
    const size_t rows = d.t.size();
    std::vector<T> t(d.t.begin(), d.t.end()), y(d.y.begin(), d.y.end()), dy(d.dy.begin(), d.dy.end());
    // objects: runs of equal ids (source/main.cu:468-510); one object in the single modes
    std::vector<size_t> start{0};
    if (a.mode == 1 || a.mode == 4)
        for (size_t i = 1; i < rows; ++i)
            if (d.id[i] != d.id[i - 1]) start.push_back(i);
    const size_t nobj = start.size();
    const size_t nf = (size_t)a.nfreq;
    std::vector<T> pgram(nobj * nf, T(0));
    printf("\nDataset file: %s", a.file.c_str());
    printf("\nData import: Total rows: %zu", rows);
    const auto t0 = std::chrono::steady_clock::now();
    fn(d.id.data(), t.data(), y.data(), dy.data(), (unsigned)rows, a.fmin, a.fmax, (unsigned)nf,
       a.mode, pgram.data());
    fflush(stdout);
    const double secs =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st() != 0) {
        fprintf(stderr, "lsgb_main: LombScarglePy failed with status %d\n", st());
        return 1;
    }
    // periods from the periodogram, first maximum from power 0 (source/main.cu:1545-1563)
    const T fminT = (T)a.fmin, fmaxT = (T)a.fmax;
    const double step = (double)(T)(((double)fmaxT - (double)fminT) / (nf * 1.0));
    std::vector<double> per(3 * nobj), pow3(3 * nobj);
    double sum = 0;
    for (size_t o = 0; o < nobj; ++o) {
        const T *p = pgram.data() + o * nf;
        size_t best[3] = {0, 0, 0};
        T bp[3] = {0, 0, 0};
        for (int r = 0; r < 3; ++r)  // three scans, each skipping the earlier maxima (:1165-1219)
            for (size_t k = 0; k < nf; ++k) {
                bool skip = false;
                for (int q = 0; q < r; ++q) skip |= (k == best[q]);
                if (!skip && bp[r] < p[k]) {
                    bp[r] = p[k];
                    best[r] = k;
                }
            }
        for (int r = 0; r < 3; ++r) {
            per[3 * o + r] = (1.0 / ((double)fminT + best[r] * step)) * 2.0 * M_PI;
            pow3[3 * o + r] = (double)bp[r];
        }
        sum += per[3 * o];
    }
    const uint32_t single_id = d.id.empty() ? 0 : d.id[0];
    auto obj_id = [&](size_t o) { return (a.mode == 2 || a.mode == 5) ? single_id : d.id[start[o]]; };
    if (!a.quiet) printf("\nTotal time: %f", secs);
    printf("\n[lsgb_main] Sum of periods: %f\n", sum);
    if (a.print_screen)
        for (size_t o = 0; o < nobj; ++o)
            printf("Object: %u Period: %f, Power: %f \n", obj_id(o), per[3 * o], pow3[3 * o]);
    if (!a.period_file.empty()) {
        std::ofstream f(a.period_file);
        f.precision(6);
        for (size_t o = 0; o < nobj; ++o) f << obj_id(o) << ", " << per[3 * o] << ", " << pow3[3 * o] << "\n";
    }
    if (!a.top3_file.empty()) {
        std::ofstream f(a.top3_file);
        f.precision(6);
        for (size_t o = 0; o < nobj; ++o)
            f << obj_id(o) << ", " << per[3 * o] << ", " << per[3 * o + 1] << ", " << per[3 * o + 2]
              << ", " << pow3[3 * o] << ", " << pow3[3 * o + 1] << ", " << pow3[3 * o + 2] << "\n";
    }
    if (!a.pgram_file.empty()) {
        std::ofstream f(a.pgram_file);
        f.precision(4);
        for (size_t o = 0; o < nobj; ++o) {
            f << obj_id(o) << ", ";
            for (size_t k = 0; k < nf; ++k) f << pgram[o * nf + k] << ", ";
            f << "\n";
        }
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
