// tcp_drive.cpp -- the reference's main program (main.f90) on top of the C ABI
// of libtcpgpu.so: reads tcp.prm and input.xyz / restart.xyz in the reference's
// formats, runs the MD loop on one GPU, and writes ener*.dat (SAMPLING),
// RDFnnn.dat / VDFnnn.dat (DUMP) and RESTnn.xyz (Restart) as result.f90 does.
//
//   tcp_drive [options] [run-directory]
//     --precision fp32c|fp64   pair arithmetic (default fp32c)
//     --ei deutsch|kelbg|coulomb  e-i model (default deutsch = the reference)
//     --lambda L               Kelbg length in A (default rs of tcp.prm)
//     --alpha A                Ewald alpha in 1/A (default 3.1/rc, force.f90:23)
//     --order P                B-spline order (default 4, force.f90:703-738)
//     --period N               apply ISOKIN/BEREND every N-th step (default 1)
//     --seed S                 seed of the Vinit velocities and STOCH noise
//     --no-rdf                 skip RDF/VDF accumulation (DUMP writes zeros)
//
// Differences from the reference driver: one GPU instead of MPI ranks; with
// rest = 'OFF' the Vinit velocities (init.f90:26-112: uniform in [-0.5, 0.5),
// mean removed, rescaled to Te / Ti) come from a seeded generator instead of
// the compiler's RANDOM_NUMBER; STOCH noise is Philox-based (vverlet.f90:390
// uses the compiler RNG), so only its statistics can match.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "tcp_gpu.h"

namespace {

constexpr double kEps = 14.399644154020082;   // data.f90:21
constexpr double kTps = 10.180505306645389;   // data.f90:22
constexpr double kPi = 3.1415926535897931;
constexpr int kNdist = 500;

[[noreturn]] void stop(const std::string &msg) {
    std::fprintf(stderr, " *** %s ***\n", msg.c_str());
    std::exit(1);
}

void check(int rc, const char *where) {
    if (rc != TCP_OK) stop(std::string(where) + ": " + tcp_status_string(rc) + ": " + tcp_last_error());
}

// Fortran list-directed READ of one record: the whitespace/comma separated
// tokens of the next line.
struct Records {
    std::ifstream in;
    std::string path;
    explicit Records(const std::string &p) : in(p), path(p) {
        if (!in) stop("CANNOT OPEN " + p);
    }
    std::vector<std::string> next() {
        std::string line;
        if (!std::getline(in, line)) stop("unexpected end of " + path);
        for (char &ch : line)
            if (ch == ',') ch = ' ';
        std::istringstream ss(line);
        std::vector<std::string> t;
        std::string w;
        while (ss >> w) t.push_back(w);
        return t;
    }
    double num(const std::string &s) {
        std::string t = s;
        for (char &ch : t)
            if (ch == 'd' || ch == 'D') ch = 'e';   // Fortran D exponents
        return std::strtod(t.c_str(), nullptr);
    }
};

// Fortran ESw.d edit descriptor (one digit before the point; a three-digit
// exponent drops the E as Fortran does).
std::string es(double v, int w, int d) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.*E", d, v);
    std::string s(buf);
    const size_t e = s.find('E');
    const int ex = std::atoi(s.c_str() + e + 1);
    if (std::abs(ex) > 99) s = s.substr(0, e) + (ex < 0 ? "-" : "+") + std::to_string(std::abs(ex));
    if ((int)s.size() < w) s = std::string(w - s.size(), ' ') + s;
    return s;
}

struct Particle {
    double x[3], v[3], f[3];
    int id;
};

// splitmix64 -> uniform doubles in [0, 1)
struct Rng {
    uint64_t s;
    double uniform() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
};

}  // namespace

int main(int argc, char **argv) {
    std::string dir = ".", precision = "fp32c", ei = "deutsch";
    double lambda = -1, alpha = -1;
    int order = 4, period = 1;
    uint64_t seed = 1;
    bool rdf_on = true;
    for (int k = 1; k < argc; ++k) {
        std::string a = argv[k];
        auto val = [&]() -> std::string {
            if (k + 1 >= argc) stop("missing value for " + a);
            return argv[++k];
        };
        if (a == "--precision") precision = val();
        else if (a == "--ei") ei = val();
        else if (a == "--lambda") lambda = std::atof(val().c_str());
        else if (a == "--alpha") alpha = std::atof(val().c_str());
        else if (a == "--order") order = std::atoi(val().c_str());
        else if (a == "--period") period = std::atoi(val().c_str());
        else if (a == "--seed") seed = std::strtoull(val().c_str(), nullptr, 10);
        else if (a == "--no-rdf") rdf_on = false;
        else if (a[0] == '-') stop("unknown option " + a);
        else dir = a;
    }
    const auto t_wall0 = std::chrono::steady_clock::now();

    // ---- tcp.prm, main.f90:221-294 -----------------------------------------
    Records prm(dir + "/tcp.prm");
    tcp_params p;
    std::memset(&p, 0, sizeof p);
    prm.next();
    prm.next();
    auto t = prm.next();
    if (t.size() < 5) stop("tcp.prm: time line needs tmax trest tdump tsamp dt");
    double tmax = prm.num(t[0]) / kTps, trest = prm.num(t[1]) / kTps, tdump = prm.num(t[2]) / kTps,
           tsamp = prm.num(t[3]) / kTps, dt = prm.num(t[4]) / kTps;            // main.f90:232-237
    prm.next();
    t = prm.next();
    for (int d = 0; d < 3; ++d) p.box[d] = prm.num(t.at(d));
    prm.next();
    p.Te = prm.num(prm.next().at(0));
    p.Ti = prm.num(prm.next().at(0));
    prm.next();
    const int ntel = std::atoi(prm.next().at(0).c_str());
    const int ntion = std::atoi(prm.next().at(0).c_str());
    prm.next();
    p.rc = prm.num(prm.next().at(0));
    prm.next();
    p.rs = prm.num(prm.next().at(0));
    prm.next();
    p.xm[0] = prm.num(prm.next().at(0));
    p.xm[1] = prm.num(prm.next().at(0));
    prm.next();
    p.q[0] = prm.num(prm.next().at(0));
    p.q[1] = prm.num(prm.next().at(0));
    prm.next();
    std::string thermo = prm.next().at(0);
    t = prm.next();
    p.tau = prm.num(t.at(0));
    p.alpha_lgv = prm.num(t.at(1));
    prm.next();
    t = prm.next();
    const std::string rest = t.at(0);
    prm.next();
    t = prm.next();
    p.dx_ee = prm.num(t.at(0));
    p.dx_ei = prm.num(t.at(1));
    p.dx_ii = prm.num(t.at(2));
    p.dv_e = p.Te * 4.0 / kNdist;                                             // main.f90:286-287
    p.dv_i = p.Ti * 4.0 / kNdist;
    prm.next();
    t = prm.next();
    for (int d = 0; d < 3; ++d) p.K[d] = std::atoi(t.at(d).c_str());
    for (char &ch : thermo) ch = (char)std::toupper((unsigned char)ch);
    if (thermo.rfind("STOCH", 0) == 0) p.thermo = TCP_THERMO_STOCH;
    else if (thermo == "BEREND") p.thermo = TCP_THERMO_BEREND;
    else if (thermo == "ISOKIN") p.thermo = TCP_THERMO_ISOKIN;
    else p.thermo = TCP_THERMO_NOTEMP;
    p.a = alpha;
    p.order = order;
    p.ei_model = ei == "kelbg" ? TCP_EI_KELBG : (ei == "coulomb" ? TCP_EI_COULOMB : TCP_EI_DEUTSCH);
    p.lambda_ei = lambda > 0 ? lambda : p.rs;
    p.charge_scale = 1.0;
    p.precision = precision == "fp64" ? TCP_PREC_FP64 : TCP_PREC_FP32C;
    p.reciprocal = TCP_RECIP_SPME;
    p.thermo_period = period;
    p.seed = seed;

    // ---- particles: input.xyz (main.f90:347-379) or restart.xyz (:383-441) ----
    std::vector<Particle> el(ntel), io(ntion);
    const bool from_restart = rest != "OFF";
    {
        Records xyz(dir + (from_restart ? "/restart.xyz" : "/input.xyz"));
        xyz.next();
        xyz.next();
        for (auto *arr : {&el, &io})
            for (auto &q : *arr) {
                auto r = xyz.next();
                if (from_restart) {
                    if (r.size() < 11) stop("restart.xyz: record needs name x y z vx vy vz fx fy fz id");
                    for (int d = 0; d < 3; ++d) {
                        q.x[d] = xyz.num(r[1 + d]);
                        q.v[d] = xyz.num(r[4 + d]);
                        q.f[d] = xyz.num(r[7 + d]);
                    }
                    q.id = std::atoi(r[10].c_str());
                } else {
                    if (r.size() < 5) stop("input.xyz: record needs name x y z id");
                    for (int d = 0; d < 3; ++d) q.x[d] = xyz.num(r[1 + d]);
                    q.id = std::atoi(r[4].c_str());
                }
            }
    }
    // Vinit (init.f90:26-112) with a seeded generator
    if (!from_restart) {
        Rng rng{seed};
        for (int s = 0; s < 2; ++s) {
            auto &arr = s == 0 ? el : io;
            if (arr.empty()) continue;
            double mean[3] = {0, 0, 0};
            for (auto &q : arr)
                for (int d = 0; d < 3; ++d) mean[d] += (q.v[d] = rng.uniform() - 0.5);
            double mv2 = 0.0;
            for (auto &q : arr)
                for (int d = 0; d < 3; ++d) {
                    q.v[d] -= mean[d] / arr.size();
                    mv2 += p.xm[s] * q.v[d] * q.v[d];
                }
            const double lam = std::sqrt((s == 0 ? p.Te : p.Ti) / (mv2 / (3.0 * arr.size())));
            for (auto &q : arr)
                for (int d = 0; d < 3; ++d) q.v[d] *= lam;
        }
    }

    tcp_ctx *ctx = nullptr;
    check(tcp_create(&p, ntel, ntion, 0, &ctx), "tcp_create");
    double a_out = 0, uo = 0;
    check(tcp_ewald_self(ctx, &a_out, &uo), "EWALD_SELF");                    // main.f90:46
    const long stride = sizeof(Particle);
    if (ntel) check(tcp_upload(ctx, 0, el[0].x, el[0].v, el[0].f, stride), "tcp_upload");
    if (ntion) check(tcp_upload(ctx, 1, io[0].x, io[0].v, io[0].f, stride), "tcp_upload");
    tcp_energies e{};
    if (!from_restart) check(tcp_finit(ctx, dt, &e), "Finit");                // main.f90:52
    check(tcp_set_flags(ctx, TCP_FLAG_ENERGY | (rdf_on ? TCP_FLAG_RDF | TCP_FLAG_VDF : 0u)), "tcp_set_flags");

    // ---- main loop, main.f90:57-170 -----------------------------------------
    const long ndump = std::lround(tdump / dt), nrest = std::lround(trest / dt), nsamp = std::lround(tsamp / dt);
    const long nloop_max = std::lround(tmax / dt);
    const double V = p.box[0] * p.box[1] * p.box[2];
    std::FILE *ener = std::fopen((dir + "/ener00.dat").c_str(), "w");
    const char *ener_header =
        "# time(fs),       T_el(eV),      T_ion(eV), Potential Energy,  Total energy, Electron VAF, Ion VAF,  mutual VAF\n";
    std::fputs(ener_header, ener);
    std::vector<double> rdf(3 * (kNdist + 1)), vdf(2 * (kNdist + 1));
    double tnow = 0.0;
    long nloop = 0;
    double gpu_s = 0.0;
    while (nloop < nloop_max) {
        // run up to the next output event in one call
        long next = nloop_max;
        for (long per : {ndump, nsamp, nrest})
            if (per > 0) next = std::min(next, (nloop / per + 1) * per);
        const int nsteps = (int)(next - nloop);
        const auto g0 = std::chrono::steady_clock::now();
        check(tcp_md_steps(ctx, dt, nsteps, &e), "tcp_md_steps");
        gpu_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - g0).count();
        nloop = next;
        tnow += nsteps * dt;
        if (ndump > 0 && nloop % ndump == 0) {                                  // DUMP, result.f90:209-278
            check(tcp_histograms(ctx, rdf.data(), vdf.data(), 1), "tcp_histograms");
            const long nfreq = nloop / ndump;
            const double ntau = (double)ndump;
            char name[64];
            std::snprintf(name, sizeof name, "/RDF%03ld.dat", nfreq);
            std::FILE *fr = std::fopen((dir + name).c_str(), "w");
            std::fputs("#  x_ee,      RDF_ee,      x_ei    RDF_ei,       x_ii     RDF_ii\n", fr);
            const double ntpt = (double)(ntel + ntion);
            const double dvee = (double)ntel * ntel * ntau * std::pow(p.dx_ee, 3) * 4. * kPi / 3.0 / V;
            const double dvei = ntpt * ntpt * ntau * std::pow(p.dx_ei, 3) * 4. * kPi / 3.0 / V;
            const double dvii = (double)ntion * ntion * ntau * std::pow(p.dx_ii, 3) * 4. * kPi / 3.0 / V;
            for (int i = 1; i <= kNdist; ++i) {
                const double sh = (double)i * i * i - (double)(i - 1) * (i - 1) * (i - 1);
                std::fprintf(fr, "%s %s %s %s %s %s \n", es(i * p.dx_ee, 14, 6).c_str(),
                             es(rdf[i - 1] / dvee / sh, 14, 6).c_str(), es(i * p.dx_ei, 14, 6).c_str(),
                             es(rdf[(kNdist + 1) + i - 1] / dvei / sh, 14, 6).c_str(), es(i * p.dx_ii, 14, 6).c_str(),
                             es(rdf[2 * (kNdist + 1) + i - 1] / dvii / sh, 14, 6).c_str());
            }
            std::fclose(fr);
            std::snprintf(name, sizeof name, "/VDF%03ld.dat", nfreq);
            std::FILE *fv = std::fopen((dir + name).c_str(), "w");
            std::fputs("#  T_e        VDF_e            T_i      VDF_i\n", fv);
            for (int i = 1; i <= kNdist; ++i)
                std::fprintf(fv, "%s %s %s %s \n", es(p.dv_e * i, 14, 6).c_str(), es(vdf[i - 1] / ntau, 14, 6).c_str(),
                             es(p.dv_i * i, 14, 6).c_str(), es(vdf[(kNdist + 1) + i - 1] / ntau, 14, 6).c_str());
            std::fclose(fv);
        }
        if (nsamp > 0 && nloop % nsamp == 0) {                                  // SAMPLING, result.f90:298-320
            const double epot = e.Um + e.Epot;
            std::fprintf(ener, "%s %s %s %s %s \n", es(tnow * kTps, 15, 8).c_str(), es(e.mv2el / (3.0 * ntel), 15, 8).c_str(),
                         es(e.mv2ion / (3.0 * ntion), 15, 8).c_str(), es(epot, 15, 8).c_str(),
                         es(0.5 * (e.mv2el + e.mv2ion) + epot, 15, 8).c_str());
            std::fflush(ener);
        }
        if (nrest > 0 && nloop % nrest == 0) {                                  // Restart, result.f90:3-134
            if (ntel) check(tcp_download(ctx, 0, el[0].x, el[0].v, el[0].f, stride), "tcp_download");
            if (ntion) check(tcp_download(ctx, 1, io[0].x, io[0].v, io[0].f, stride), "tcp_download");
            const long nfreq = nloop / nrest;
            char name[64];
            std::snprintf(name, sizeof name, "/REST%02ld.xyz", nfreq);
            std::FILE *fo = std::fopen((dir + name).c_str(), "w");
            std::fprintf(fo, " %11d\n frame = %11ld energy = 0\n", ntel + ntion, nfreq);
            for (int s = 0; s < 2; ++s)
                for (auto &q : s == 0 ? el : io) {
                    std::fprintf(fo, "%-3s", s == 0 ? "Cu" : "C");
                    for (double v : {q.x[0], q.x[1], q.x[2], q.v[0], q.v[1], q.v[2], q.f[0], q.f[1], q.f[2]})
                        std::fprintf(fo, " %s", es(v, 14, 6).c_str());
                    std::fprintf(fo, " %6d\n", q.id);
                }
            std::fclose(fo);
            std::fclose(ener);
            std::snprintf(name, sizeof name, "/ener%02ld.dat", nfreq);
            ener = std::fopen((dir + name).c_str(), "w");
            std::fputs(ener_header, ener);
        }
    }
    std::fclose(ener);
    tcp_destroy(ctx);
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_wall0).count();
    std::printf("  Wall time is %8.2f\n", wall);                                // main.f90:184-186
    std::printf("  md steps (GPU) = %8.2f s, %ld steps\n", gpu_s, nloop);
    return 0;
}
