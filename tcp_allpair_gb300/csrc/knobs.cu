// knobs.cu -- the GPU build's own parameters for callers that fill
// tcp_params from the reference's input (tcp.prm, main.f90:221-294), which
// has no field for them: the precision, the e-i model, the spline order, an
// explicit Ewald alpha, the Kelbg length, the reciprocal method and the
// device.  tcp_params_from_env() reads them from an optional file and from
// environment variables (see include/tcp_gpu.h); the Fortran drop-in module
// calls it in EWALD_SELF before creating the context.  Host code only.
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "tcp_internal.h"

namespace tcp {
namespace {

std::string lower(std::string s) {
    for (char &ch : s) ch = (char)std::tolower((unsigned char)ch);
    return s;
}

std::string upper(std::string s) {
    for (char &ch : s) ch = (char)std::toupper((unsigned char)ch);
    return s;
}

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

bool to_long(const std::string &v, long long &out) {
    if (v.empty()) return false;
    char *end = nullptr;
    errno = 0;
    const long long x = std::strtoll(v.c_str(), &end, 10);
    if (errno || !end || *end) return false;
    out = x;
    return true;
}

bool to_double(const std::string &v, double &out) {
    if (v.empty()) return false;
    std::string w = v;
    for (char &ch : w)   // Fortran exponents: 1.0D-3
        if (ch == 'd' || ch == 'D') ch = 'e';
    char *end = nullptr;
    errno = 0;
    const double x = std::strtod(w.c_str(), &end);
    if (errno || !end || *end) return false;
    out = x;
    return true;
}

// value as one of names[] (case-insensitive) or its index
bool to_enum(const std::string &v, const char *const *names, int count, int &out) {
    const std::string l = lower(v);
    for (int k = 0; k < count; ++k)
        if (l == names[k]) {
            out = k;
            return true;
        }
    long long x;
    if (to_long(v, x) && x >= 0 && x < count) {
        out = (int)x;
        return true;
    }
    return false;
}

const char *const kKeys[] = {"precision", "ei_model", "reciprocal", "order", "alpha", "lambda_ei",
                             "ewald_nmax2", "thermo_period", "seed", "charge_scale", "device", "sync_every"};

int apply(tcp_params *p, int *device, int *sync_every, const std::string &key, const std::string &val,
          const std::string &where) {
    static const char *const prec[] = {"fp64", "fp32c", "fp32c_r64"};
    static const char *const ei[] = {"deutsch", "kelbg", "coulomb"};
    static const char *const recip[] = {"none", "spme", "ewald"};
    auto bad = [&](const char *what) {
        return set_error(TCP_ERR_BAD_PARAM, where + ": " + key + " = '" + val + "': " + what);
    };
    long long n = 0;
    double d = 0.0;
    int e = 0;
    if (key == "precision") {
        if (!to_enum(val, prec, 3, e)) return bad("expected fp64, fp32c or fp32c_r64");
        p->precision = e;
    } else if (key == "ei_model") {
        if (!to_enum(val, ei, 3, e)) return bad("expected deutsch, kelbg or coulomb");
        p->ei_model = e;
    } else if (key == "reciprocal") {
        if (!to_enum(val, recip, 3, e)) return bad("expected none, spme or ewald");
        p->reciprocal = e;
    } else if (key == "order") {
        if (!to_long(val, n) || n < 4 || n > kMaxOrder) return bad("expected an integer in 4..8");
        p->order = (int)n;
    } else if (key == "alpha") {
        if (!to_double(val, d) || !(d >= 0.0)) return bad("expected a number >= 0 (0: 3.1/rc)");
        p->a = d;
    } else if (key == "lambda_ei") {
        if (!to_double(val, d) || !(d > 0.0)) return bad("expected a length > 0");
        p->lambda_ei = d;
    } else if (key == "ewald_nmax2") {
        if (!to_long(val, n) || n < 0 || n > 1000000) return bad("expected an integer >= 0");
        p->ewald_nmax2 = (int)n;
    } else if (key == "thermo_period") {
        if (!to_long(val, n) || n < 1 || n > 1000000000) return bad("expected an integer >= 1");
        p->thermo_period = (int)n;
    } else if (key == "seed") {
        if (!to_long(val, n) || n < 0) return bad("expected an integer >= 0");
        p->seed = (uint64_t)n;
    } else if (key == "charge_scale") {
        if (!to_double(val, d) || !(d > 0.0)) return bad("expected a number > 0");
        p->charge_scale = d;
    } else if (key == "device") {
        if (!to_long(val, n) || n < 0 || n > 1024) return bad("expected a device index");
        if (device) *device = (int)n;
    } else if (key == "sync_every") {
        if (!to_long(val, n) || n < 0 || n > 1000000000) return bad("expected an integer >= 0");
        if (sync_every) *sync_every = (int)n;
    } else {
        return set_error(TCP_ERR_BAD_PARAM, where + ": unknown key '" + key + "'");
    }
    return TCP_OK;
}

}  // namespace
}  // namespace tcp

extern "C" int tcp_params_from_env(tcp_params *p, int *device, int *sync_every) {
    using namespace tcp;
    if (!p) return set_error(TCP_ERR_BAD_PARAM, "params is NULL");
    std::vector<std::pair<std::string, std::string>> kv;   // (key, value), later entries win
    std::vector<std::string> origin;
    const char *env_path = std::getenv("TCP_GPU_PRM");
    const std::string path = env_path ? env_path : "tcp_gpu.prm";
    if (FILE *f = std::fopen(path.c_str(), "r")) {
        char line[1024];
        int lineno = 0;
        while (std::fgets(line, sizeof line, f)) {
            ++lineno;
            std::string s(line);
            const size_t hash = s.find_first_of("#!");
            if (hash != std::string::npos) s.resize(hash);
            s = trim(s);
            if (s.empty()) continue;
            size_t sep = s.find('=');
            if (sep == std::string::npos) sep = s.find_first_of(" \t");
            if (sep == std::string::npos) {
                std::fclose(f);
                return set_error(TCP_ERR_BAD_PARAM, path + ":" + std::to_string(lineno) + ": expected 'key value'");
            }
            kv.emplace_back(lower(trim(s.substr(0, sep))), trim(s.substr(sep + 1)));
            origin.push_back(path + ":" + std::to_string(lineno));
        }
        std::fclose(f);
    } else if (env_path) {
        return set_error(TCP_ERR_BAD_PARAM, "TCP_GPU_PRM=" + path + " cannot be opened");
    }
    for (const char *k : kKeys) {
        const std::string name = "TCP_GPU_" + upper(k);
        if (const char *v = std::getenv(name.c_str())) {
            kv.emplace_back(k, trim(v));
            origin.push_back(name);
        }
    }
    for (size_t i = 0; i < kv.size(); ++i)
        if (int rc = apply(p, device, sync_every, kv[i].first, kv[i].second, origin[i])) return rc;
    return TCP_OK;
}
