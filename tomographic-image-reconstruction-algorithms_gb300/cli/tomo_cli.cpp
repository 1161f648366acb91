// tomo_cli.cpp -- the reference's command-line drivers on top of libtomo.so.
//
// Each executable keeps its reference counterpart's positional arguments,
// input files and output files; the hot path is one tomo_iterate call per
// iteration.  Compiled once per driver with -DTOMO_DRIVER_<NAME>; the `tomo`
// executable takes the driver name as its first argument.
//
//   generate-field [--binary]                       generate-field.cu:45-113
// A phantom named *.bin selects the binary file form (cli/textio.h) for the
// data files and the image a run writes; reading accepts either form.
//   generate-data <fo> <gs> [<noise %>]              generate-data.cu:57-224
//   sirt-mimo <gs> <eps> <iters> <omega>             sirt-mimo.cu:66-387
//   sirt-mimo-io <fo> <gs> <eps> <iters> <w> <a> <b> <g>      sirt-mimo-io.cu
//   sirt-mimo-norm <fo> <gs> <eps> <iters> <w> <a> <b> <g>    sirt-mimo-norm.cu:122-512
//   sirt-mimo-norm-mem <fo> <gs> <P> <eps> <iters> <w> <a> <b> <g>  sirt-mimo-norm-mem.cu:125-146
//   sirt-mimo-weight <fo> <gs> <eps> <iters> <a> <b> <w>      sirt-mimo-weight.cu:69
//   sirt-mimo-avg <fo> <gs> <eps> <iters>                     sirt-mimo-avg.cu:114
//   sirt-mimo-avg-weight <fo> <gs> <eps> <iters>              sirt-mimo-avg-weight.cu
//   sirt-iter <fo> <gs> <eps> <iters> <w> <a>                 sirt-iter.cu:411-437
//   sirt-iter-norm <fo> <gs> <eps> <iters> <w> <a>            sirt-iter-norm.cu
//   art-mimo <gs> <eps> <iters> <omega>                       art-mimo.cu:480-788
//   art-mimo-io <fo> <gs> <eps> <iters> <w> <a> <b> <g>       art-mimo-io.cu
//   sirt-mimo-seq <fo> <gs> <eps> <iters> <w> <a> <b> <g>     sirt-mimo-seq.cu:34,337-596
//       (5 ART iterations, then normalised SIRT; one schedule, iteration index continues)
//   sirt-mimo-norm-alt <fo> <gs> <P> <eps> <iters> <a1> <b1> <n1> <a2> <b2> <n2>
//       sirt-mimo-norm-alt.cu:126-156,421-477 (normalised SIRT, scale alternating between
//       a1 + b1/k^n1 on odd and a2 - b2/k^n2 on even 1-based iterations k; a, b x 1000)
// max iterations -1 means unbounded (sirt-mimo.cu:79-80).  Data files are
// <base>-data-{bottom,right,top,left}-<gs>.txt (generate-data.cu:197-223).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <string>
#include <vector>

#include "textio.h"
#include "tomo.h"

namespace {

const char* kSides[4] = {"bottom", "right", "top", "left"};

int die(const char* msg) {
    std::fprintf(stderr, "Error: %s\n\n", msg);
    return 1;
}

int check(tomo_status s, tomo_ctx* c, const char* what) {
    if (s == TOMO_OK) return 0;
    std::fprintf(stderr, "Error: %s: %s (%s)\n", what, tomo_status_string(s), tomo_last_error(c));
    return 1;
}

bool parse_int(const char* s, int* out) {
    char* e = nullptr;
    const long v = std::strtol(s, &e, 10);
    if (e == s || *e) return false;
    *out = (int)v;
    return true;
}

bool parse_float(const char* s, float* out) {
    char* e = nullptr;
    const float v = std::strtof(s, &e);
    if (e == s || *e) return false;
    *out = v;
    return true;
}

// Extension of every file a run writes: the phantom's (".txt", or ".bin" for the binary form).
std::string g_ext = ".txt";

// "<base>.<ext>" with exactly one period (generate-data.cu:68-73); sets the run's file form
bool split_base(const std::string& fo, std::string* base) {
    if (std::count(fo.begin(), fo.end(), '.') != 1) return false;
    *base = fo.substr(0, fo.find('.'));
    g_ext = textio::is_binary_name(fo) ? ".bin" : ".txt";
    return true;
}

std::string data_name(const std::string& base, int side, int gs) {
    return base + "-data-" + kSides[side] + "-" + std::to_string(gs) + g_ext;
}

// records rec[g][k][side*nx + i]  <->  four files side[g][k][i]
bool write_records(const std::string& base, int gs, const std::vector<float>& rec, int G, int nt, int nx) {
    std::vector<float> side((size_t)G * nt * nx);
    for (int s = 0; s < 4; ++s) {
        for (int g = 0; g < G; ++g)
            for (int k = 0; k < nt; ++k)
                std::memcpy(&side[((size_t)g * nt + k) * nx], &rec[((size_t)g * nt + k) * 4 * nx + (size_t)s * nx],
                            sizeof(float) * nx);
        const std::string name = data_name(base, s, gs);
        std::fprintf(stderr, "writing to '%s'...\n\n", name.c_str());
        if (!textio::write_floats(name, side.data(), nx, nt, G)) return false;
    }
    return true;
}

bool read_records(const std::string& base, int gs, std::vector<float>& rec, int G, int nt, int nx) {
    std::vector<float> side((size_t)G * nt * nx);
    rec.assign((size_t)G * nt * 4 * nx, 0.f);
    for (int s = 0; s < 4; ++s) {
        const std::string name = data_name(base, s, gs);
        if (!textio::read_floats(name, side.data(), side.size())) {
            std::fprintf(stderr, "Error: '%s' file not found in current directory.\n\n", name.c_str());
            return false;
        }
        for (int g = 0; g < G; ++g)
            for (int k = 0; k < nt; ++k)
                std::memcpy(&rec[((size_t)g * nt + k) * 4 * nx + (size_t)s * nx], &side[((size_t)g * nt + k) * nx],
                            sizeof(float) * nx);
    }
    return true;
}

struct Problem {
    tomo_config cfg{};
    tomo_ctx* ctx = nullptr;
    tomo_info info{};
    std::vector<float> fo, rec;
    ~Problem() { tomo_destroy(ctx); }
};

int open_problem(Problem& p, int gs, int groups_per_pass) {
    tomo_config_init(&p.cfg, TOMO_PROFILE_REF);
    p.cfg.group_size = gs;
    p.cfg.groups_per_pass = groups_per_pass;
    if (const char* d = std::getenv("TOMO_DEVICE")) p.cfg.device = std::atoi(d);
    if (check(tomo_create(&p.cfg, &p.ctx), nullptr, "tomo_create")) return 1;
    tomo_get_info(p.ctx, &p.info);
    return 0;
}

// Loads fo.txt-style phantom and its four data files.
int load_inputs(Problem& p, const std::string& fo_name, int gs, std::string* base) {
    if (!split_base(fo_name, base)) {
        std::fprintf(stderr, "Error: '%s' should have only one period.\n", fo_name.c_str());
        return 1;
    }
    const int nx = p.cfg.nx, ny = p.cfg.ny;
    p.fo.assign((size_t)nx * ny, 0.f);
    if (!textio::read_floats(fo_name, p.fo.data(), p.fo.size())) {
        std::fprintf(stderr, "Error: '%s' file not found in current directory.\n\n", fo_name.c_str());
        return 1;
    }
    if (!read_records(*base, gs, p.rec, p.info.n_groups, p.cfg.nt, nx)) return 1;
    return check(tomo_set_records(p.ctx, p.rec.data()), p.ctx, "tomo_set_records");
}

// Generates the reference phantom and its data in-process (sirt-mimo.cu:127-206).
int self_generate(Problem& p) {
    const int nx = p.cfg.nx, ny = p.cfg.ny;
    p.fo.assign((size_t)nx * ny, 0.f);
    if (check(tomo_phantom_ref(nx, ny, p.fo.data()), nullptr, "tomo_phantom_ref")) return 1;
    p.rec.assign((size_t)p.info.n_groups * p.cfg.nt * p.info.n_channels, 0.f);
    if (check(tomo_forward(p.ctx, p.fo.data(), p.rec.data(), nullptr), p.ctx, "tomo_forward")) return 1;
    return check(tomo_set_records(p.ctx, p.rec.data()), p.ctx, "tomo_set_records");
}

struct LoopOpts {
    int method;
    tomo_schedule sched;
    float target;
    int max_iters;
    bool table;              // sirt-mimo-norm style table vs sirt-mimo style lines
    bool abs_threshold;      // |file_eps - eps| > 0.2 (norm) vs file_eps - eps > 0.2 (classic)
    const char* conv_name;   // sirt_convergence.txt / art_convergence.txt
    const char* time_name;
    // optional per-iteration method and schedule (hybrid and alternating drivers)
    std::function<int(int)> method_at = {};
    std::function<tomo_schedule(int)> sched_at = {};
};

// The iteration loop with the reference's stopping rule and log files.
int iterate_loop(Problem& p, const LoopOpts& o, std::vector<float>& f) {
    const int nx = p.cfg.nx, ny = p.cfg.ny;
    f.assign((size_t)nx * ny, 0.f);
    FILE* conv = std::fopen(o.conv_name, "w");
    FILE* tfile = std::fopen(o.time_name, "w");
    const int64_t limit = o.max_iters < 0 ? std::numeric_limits<int>::max() : o.max_iters;
    float prev = o.table ? 100.f : std::numeric_limits<float>::infinity();
    float file_eps = std::numeric_limits<float>::infinity();
    if (o.table) std::printf("  iter      epsilon      difference \n------ ------------ --------------- \n");
    const auto t0 = std::chrono::steady_clock::now();
    int rc = 0;
    for (int64_t it = 0; it < limit; ++it) {
        tomo_iter_stats st{};
        const int method = o.method_at ? o.method_at((int)it) : o.method;
        const tomo_schedule sc = o.sched_at ? o.sched_at((int)it) : o.sched;
        if (check(tomo_iterate(p.ctx, method, &sc, (int)it, f.data(), nullptr, p.fo.data(), &st), p.ctx,
                  "tomo_iterate")) { rc = 1; break; }
        const float eps = (float)st.epsilon;
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        const float de = file_eps - eps;
        if ((o.abs_threshold ? std::fabs(de) : de) > 0.2f) {
            if (conv) std::fprintf(conv, "%.9g ", eps);
            if (tfile) std::fprintf(tfile, "%.9g ", secs);
            file_eps = eps;
        }
        if (o.table) std::printf("%6lld %12.9g %15.9g %.9g \n", (long long)it, eps, prev - eps, st.scale);
        else std::printf("\nIter: %lld\nepsilon = %.8f\n", (long long)it, eps);
        std::fflush(stdout);
        if (eps <= o.target) {
            std::fprintf(stderr, "reached target epsilon = %.2f, at iter = %lld, epsilon = %.8f\n\n", o.target,
                         (long long)it, eps);
            break;
        }
        if (eps > prev || std::isnan(eps)) {
            std::fprintf(stderr, "diverged at iter = %lld, epsilon = %.8f\n\n", (long long)it, eps);
            break;
        }
        prev = eps;
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::fprintf(stderr, "time (s): %.6f\n", secs);
    if (conv) std::fclose(conv);
    if (tfile) std::fclose(tfile);
    return rc;
}

tomo_schedule sched(int kind, float w, float a, float b, float g) {
    tomo_schedule s{};
    s.kind = kind; s.omega = w; s.alpha = a; s.beta = b; s.gamma = g;
    return s;
}

void usage(const char* prog, const char* args) { std::fprintf(stderr, "Usage: %s %s\n\n", prog, args); }

// ---------------------------------------------------------------------------
int cmd_generate_field(int argc, char** argv) {
    const bool binary = argc == 2 && std::strcmp(argv[1], "--binary") == 0;
    if (argc != 1 && !binary) { usage(argv[0], "[--binary]"); return 1; }
    tomo_config cfg;
    tomo_config_init(&cfg, TOMO_PROFILE_REF);
    std::vector<float> fo((size_t)cfg.nx * cfg.ny);
    if (check(tomo_phantom_ref(cfg.nx, cfg.ny, fo.data()), nullptr, "tomo_phantom_ref")) return 1;
    const char* name = binary ? "fo.bin" : "fo.txt";
    std::fprintf(stderr, "writing to '%s'...\n\n", name);
    return textio::write_floats(name, fo.data(), cfg.nx, cfg.ny) ? 0 : die("cannot write the phantom");
}

int cmd_generate_data(int argc, char** argv) {
    if (argc != 3 && argc != 4) { usage(argv[0], "<fo filename> <sensor group size> [<percent noise>]"); return 1; }
    int gs;
    float pct = 0.f;
    if (!parse_int(argv[2], &gs)) return die("bad group size");
    if (argc == 4 && !parse_float(argv[3], &pct)) return die("bad noise percentage");
    std::string base;
    if (!split_base(argv[1], &base)) return die("the fo file name should have exactly one period");
    Problem p;
    if (open_problem(p, gs, 0)) return 1;
    p.fo.assign((size_t)p.cfg.nx * p.cfg.ny, 0.f);
    if (!textio::read_floats(argv[1], p.fo.data(), p.fo.size())) return die("fo file not found in current directory");
    std::vector<float> rec((size_t)p.info.n_groups * p.cfg.nt * p.info.n_channels);
    tomo_noise nz{};
    nz.kind = pct > 0.f ? 1 : 0;
    nz.level = pct / 100.f;
    nz.seed = 1234;
    if (check(tomo_generate_data(p.ctx, p.fo.data(), rec.data(), &nz), p.ctx, "tomo_generate_data")) return 1;
    return write_records(base, gs, rec, p.info.n_groups, p.cfg.nt, p.cfg.nx) ? 0 : die("cannot write data files");
}

int cmd_self(int argc, char** argv, int method) {
    if (argc != 5) { usage(argv[0], "<sensor group size> <target epsilon> <max iterations> <omega>"); return 1; }
    int gs, iters;
    float target, omega;
    if (!parse_int(argv[1], &gs) || !parse_float(argv[2], &target) || !parse_int(argv[3], &iters) ||
        !parse_float(argv[4], &omega))
        return die("bad arguments");
    Problem p;
    if (open_problem(p, gs, method == TOMO_ART ? 1 : 0) || self_generate(p)) return 1;
    const bool art = method == TOMO_ART;
    LoopOpts o{method, sched(TOMO_SCHED_CONST, omega, 0, 0, 1), target, iters, false, false,
               art ? "art_convergence.txt" : "sirt_convergence.txt", art ? "art_time.txt" : "sirt_time.txt"};
    std::vector<float> f;
    if (iterate_loop(p, o, f)) return 1;
    if (art) {
        const std::string name = "art-" + std::to_string(gs) + "-f.txt";
        return textio::write_floats(name, f.data(), p.cfg.nx, p.cfg.ny) ? 0 : die("cannot write image");
    }
    // IO_Files (sirt-mimo.cu:389-425): one row per line
    if (!textio::write_floats("dev_f0.txt", p.fo.data(), p.cfg.nx, p.cfg.ny)) return die("cannot write dev_f0.txt");
    return textio::write_floats("dev_f.txt", f.data(), p.cfg.nx, p.cfg.ny) ? 0 : die("cannot write dev_f.txt");
}

// Drivers reading <fo> and its data files.
int cmd_io(int argc, char** argv, int method, const char* prefix, int variant) {
    // variant: 0 = <fo> <gs> <eps> <iters> <w> <a> <b> <g>
    //          1 = <fo> <gs> <P> <eps> <iters> <w> <a> <b> <g>   (norm-mem)
    //          2 = <fo> <gs> <eps> <iters> <a> <b> <w>           (weight)
    //          3 = <fo> <gs> <eps> <iters>                       (avg, avg-weight)
    //          4 = <fo> <gs> <eps> <iters> <w> <a>               (sirt-iter, linear)
    //          5 = <fo> <gs> <eps> <iters> <w> <a>               (sirt-iter-norm, gamma 1.5)
    static const int nargs[6] = {9, 10, 8, 5, 7, 7};
    static const char* forms[6] = {
        "<fo_filename> <sensor group size> <target epsilon> <max iterations> <omega> <alpha> <beta> <gamma>",
        "<fo_filename> <sensor group size> <parallel groups> <target epsilon> <max iterations> <omega> <alpha> <beta> <gamma>",
        "<fo_filename> <sensor group size> <target epsilon> <max iterations> <alpha> <beta> <omega>",
        "<fo_filename> <sensor group size> <target epsilon> <max iterations>",
        "<fo_filename> <sensor group size> <target epsilon> <max iterations> <omega> <alpha>",
        "<fo_filename> <sensor group size> <target epsilon> <max iterations> <omega> <alpha>"};
    if (argc != nargs[variant]) { usage(argv[0], forms[variant]); return 1; }
    int a = 2, gs, P = 0, iters;
    float target, w = 1.f, al = 0.f, be = 0.f, ga = 1.f;
    bool ok = parse_int(argv[a++], &gs);
    if (variant == 1) ok = ok && parse_int(argv[a++], &P);
    ok = ok && parse_float(argv[a++], &target) && parse_int(argv[a++], &iters);
    tomo_schedule s{};
    if (variant == 0 || variant == 1) {
        ok = ok && parse_float(argv[a], &w) && parse_float(argv[a + 1], &al) && parse_float(argv[a + 2], &be) &&
             parse_float(argv[a + 3], &ga);
        s = sched(TOMO_SCHED_POWER, w, al, be, ga);
    } else if (variant == 2) {
        ok = ok && parse_float(argv[a], &al) && parse_float(argv[a + 1], &be) && parse_float(argv[a + 2], &w);
        s = sched(TOMO_SCHED_POWER, w, al, be, 1.f);          // omega*(alpha + beta/(it+1))
    } else if (variant == 3) {
        s = sched(TOMO_SCHED_CONST, 20000.f, 0, 0, 1);        // fixed scale (sirt-mimo-avg.cu:71)
    } else {
        ok = ok && parse_float(argv[a], &w) && parse_float(argv[a + 1], &al);
        s = variant == 4 ? sched(TOMO_SCHED_LINEAR, w, al, 1.f - al, 1.f)      // sirt-iter.cu:429,678
                         : sched(TOMO_SCHED_POWER, w, al, 1.f - al, 1.5f);     // sirt-iter-norm.cu
    }
    if (!ok) return die("bad arguments");
    Problem p;
    std::string base;
    if (open_problem(p, gs, method == TOMO_ART ? 1 : P) || load_inputs(p, argv[1], gs, &base)) return 1;
    const bool art = method == TOMO_ART;
    LoopOpts o{method, s, target, iters, true, variant != 3,
               art ? "art_convergence.txt" : "sirt_convergence.txt", art ? "art_time.txt" : "sirt_time.txt"};
    std::vector<float> f;
    if (iterate_loop(p, o, f)) return 1;
    const std::string name = std::string(prefix) + std::to_string(gs) + "-" + base + g_ext;
    return textio::write_floats(name, f.data(), p.cfg.nx, p.cfg.ny) ? 0 : die("cannot write image");
}

// sirt-mimo-seq: INITIAL_ITERATIONS = 5 ART iterations, then normalised SIRT.
int cmd_seq(int argc, char** argv) {
    if (argc != 9) {
        usage(argv[0], "<fo_filename> <sensor group size> <target epsilon> <max iterations> <omega> <alpha> <beta> <gamma>");
        return 1;
    }
    int gs, iters;
    float target, w, al, be, ga;
    if (!parse_int(argv[2], &gs) || !parse_float(argv[3], &target) || !parse_int(argv[4], &iters) ||
        !parse_float(argv[5], &w) || !parse_float(argv[6], &al) || !parse_float(argv[7], &be) ||
        !parse_float(argv[8], &ga))
        return die("bad arguments");
    Problem p;
    std::string base;
    if (open_problem(p, gs, 0) || load_inputs(p, argv[1], gs, &base)) return 1;   // ART passes one group at a time
    LoopOpts o{TOMO_SIRT_NORM, sched(TOMO_SCHED_POWER, w, al, be, ga), target, iters, true, true,
               "sirt_convergence.txt", "sirt_time.txt", nullptr, nullptr};
    o.method_at = [](int it) { return it < 5 ? TOMO_ART : TOMO_SIRT_NORM; };
    std::vector<float> f;
    if (iterate_loop(p, o, f)) return 1;
    const std::string name = "sirt-norm-" + std::to_string(gs) + "-" + base + g_ext;
    return textio::write_floats(name, f.data(), p.cfg.nx, p.cfg.ny) ? 0 : die("cannot write image");
}

// sirt-mimo-norm-alt: normalised SIRT with the alternating relaxation scale.
int cmd_norm_alt(int argc, char** argv) {
    if (argc != 12) {
        usage(argv[0], "<fo_filename> <group size> <parallel groups> <target epsilon> <max iterations> <alpha1> "
                       "<beta1> <n1> <alpha2> <beta2> <n2>");
        return 1;
    }
    int gs, P, iters;
    float target, a1, b1, n1, a2, b2, n2;
    if (!parse_int(argv[2], &gs) || !parse_int(argv[3], &P) || !parse_float(argv[4], &target) ||
        !parse_int(argv[5], &iters) || !parse_float(argv[6], &a1) || !parse_float(argv[7], &b1) ||
        !parse_float(argv[8], &n1) || !parse_float(argv[9], &a2) || !parse_float(argv[10], &b2) ||
        !parse_float(argv[11], &n2))
        return die("bad arguments");
    a1 *= 1000.f; b1 *= 1000.f; a2 *= 1000.f; b2 *= 1000.f;     // sirt-mimo-norm-alt.cu:143-148
    Problem p;
    std::string base;
    if (open_problem(p, gs, P) || load_inputs(p, argv[1], gs, &base)) return 1;
    LoopOpts o{TOMO_SIRT_NORM, sched(TOMO_SCHED_CONST, 1.f, 0, 0, 1), target, iters, true, true,
               "sirt_convergence.txt", "sirt_time.txt", nullptr, nullptr};
    o.sched_at = [=](int it) {
        const int k = it + 1;                                   // the reference counts from 1
        const float scale = k % 2 != 0 ? a1 + b1 / std::pow((float)k, n1) : a2 - b2 / std::pow((float)k, n2);
        return sched(TOMO_SCHED_CONST, scale, 0, 0, 1);
    };
    std::vector<float> f;
    if (iterate_loop(p, o, f)) return 1;
    const std::string name = "sirt-norm-" + std::to_string(gs) + "-" + base + g_ext;
    return textio::write_floats(name, f.data(), p.cfg.nx, p.cfg.ny) ? 0 : die("cannot write image");
}

int dispatch(const std::string& name, int argc, char** argv) {
    if (name == "generate-field") return cmd_generate_field(argc, argv);
    if (name == "generate-data") return cmd_generate_data(argc, argv);
    if (name == "sirt-mimo") return cmd_self(argc, argv, TOMO_SIRT_CLASSIC);
    if (name == "art-mimo") return cmd_self(argc, argv, TOMO_ART);
    if (name == "sirt-mimo-io") return cmd_io(argc, argv, TOMO_SIRT_SCALED, "sirt-", 0);
    if (name == "sirt-mimo-norm") return cmd_io(argc, argv, TOMO_SIRT_NORM, "sirt-norm-", 0);
    if (name == "sirt-mimo-norm-mem") return cmd_io(argc, argv, TOMO_SIRT_NORM, "sirt-norm-", 1);
    if (name == "sirt-mimo-weight") return cmd_io(argc, argv, TOMO_SIRT_WEIGHT, "sirt-", 2);
    if (name == "sirt-mimo-avg") return cmd_io(argc, argv, TOMO_SIRT_AVG, "sirt-", 3);
    if (name == "sirt-mimo-avg-weight") return cmd_io(argc, argv, TOMO_SIRT_AVG_WEIGHT, "sirt-", 3);
    if (name == "sirt-iter") return cmd_io(argc, argv, TOMO_SIRT_SCALED, "sirt-", 4);
    if (name == "sirt-iter-norm") return cmd_io(argc, argv, TOMO_SIRT_NORM, "sirt-norm-", 5);
    if (name == "art-mimo-io") return cmd_io(argc, argv, TOMO_ART, "art-", 0);
    if (name == "sirt-mimo-seq") return cmd_seq(argc, argv);
    if (name == "sirt-mimo-norm-alt") return cmd_norm_alt(argc, argv);
    std::fprintf(stderr, "unknown driver '%s'\n", name.c_str());
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
#if defined(TOMO_DRIVER_TOMO_MULTI)
    if (argc < 2) {
        std::fprintf(stderr, "Usage: %s <driver> [args...]\n", argv[0]);
        return 2;
    }
    return dispatch(argv[1], argc - 1, argv + 1);
#else
    const char* name =
#if defined(TOMO_DRIVER_GENERATE_FIELD)
        "generate-field";
#elif defined(TOMO_DRIVER_GENERATE_DATA)
        "generate-data";
#elif defined(TOMO_DRIVER_SIRT_MIMO)
        "sirt-mimo";
#elif defined(TOMO_DRIVER_SIRT_MIMO_IO)
        "sirt-mimo-io";
#elif defined(TOMO_DRIVER_SIRT_MIMO_NORM)
        "sirt-mimo-norm";
#elif defined(TOMO_DRIVER_SIRT_MIMO_NORM_MEM)
        "sirt-mimo-norm-mem";
#elif defined(TOMO_DRIVER_SIRT_MIMO_WEIGHT)
        "sirt-mimo-weight";
#elif defined(TOMO_DRIVER_SIRT_MIMO_AVG)
        "sirt-mimo-avg";
#elif defined(TOMO_DRIVER_SIRT_MIMO_AVG_WEIGHT)
        "sirt-mimo-avg-weight";
#elif defined(TOMO_DRIVER_SIRT_ITER)
        "sirt-iter";
#elif defined(TOMO_DRIVER_SIRT_ITER_NORM)
        "sirt-iter-norm";
#elif defined(TOMO_DRIVER_ART_MIMO)
        "art-mimo";
#elif defined(TOMO_DRIVER_ART_MIMO_IO)
        "art-mimo-io";
#elif defined(TOMO_DRIVER_SIRT_MIMO_SEQ)
        "sirt-mimo-seq";
#elif defined(TOMO_DRIVER_SIRT_MIMO_NORM_ALT)
        "sirt-mimo-norm-alt";
#else
        "unknown";
#endif
    return dispatch(name, argc, argv);
#endif
}
