// material.cu -- tabulated dielectric functions (the reference's material.c:63-293).
//
// A material file lists xi (rad/s) and eps(i xi) in ascending xi, one pair per line,
// with Drude parameters for the extrapolation below and above the table in comment
// lines ("# omegap_low = 9.0eV", "# gamma_low = 0.03eV", "# omegap_high = ...",
// "# gamma_high = ...").  eps(i xi) - 1 is interpolated linearly inside the table and
// extrapolated as omegap^2 / (xi (xi + gamma)) outside it; parameters that a file does
// not give are 0 (eps = 1).  Host code: a material enters the GPU batch through the
// eps callbacks, evaluated once per frequency.
#include <cctype>
#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/libcaps.h"

namespace {

// the longest number at the start of s (after blanks), 0 if none, like atof
double lead_number(const char *s)
{
    while (*s == ' ') s++;
    if (*s == '+') s++;
    double v = 0.0;
    const char *end = s + std::strlen(s);
    std::from_chars(s, end, v);
    return v;
}

// "... key ... = value" -> value (the first '=' after the key), as the reference's _parse
bool parse_key(const std::string &line, const char *key, double *value)
{
    const size_t k = line.find(key);
    if (k == std::string::npos) return false;
    const size_t eq = line.find('=', k + std::strlen(key));
    if (eq == std::string::npos) return false;
    *value = lead_number(line.c_str() + eq + 1);
    return true;
}

std::string trimmed(const char *raw)
{
    std::string s(raw);
    size_t b = 0, e = s.size();
    while (b < e && std::isspace((unsigned char)s[b])) b++;
    while (e > b && std::isspace((unsigned char)s[e - 1])) e--;
    s = s.substr(b, e - b);
    for (char &c : s)
        if (c == '\t') c = ' ';
    return s;
}

} // namespace

extern "C" material_t *material_init(const char *filename, double calL)
{
    FILE *f = std::fopen(filename, "r");
    if (!f) return nullptr;
    material_t *m = (material_t *)std::calloc(1, sizeof(material_t));
    m->calL = calL;
    std::strncpy(m->filename, filename, sizeof(m->filename) - 1);
    std::vector<double> xs, es;
    char buf[2048];
    bool ok = true;
    while (std::fgets(buf, sizeof buf, f)) {
        const std::string line = trimmed(buf);
        if (!line.empty() && line[0] == '#') {
            parse_key(line, "omegap_low", &m->omegap_low);
            parse_key(line, "gamma_low", &m->gamma_low);
            parse_key(line, "omegap_high", &m->omegap_high);
            parse_key(line, "gamma_high", &m->gamma_high);
            continue;
        }
        const size_t sp = line.find(' ');
        if (sp == std::string::npos) continue;
        const double xi = lead_number(line.c_str()), epsm1 = lead_number(line.c_str() + sp) - 1;
        if (!xs.empty() && xi <= xs.back()) { ok = false; break; } // frequencies must ascend
        xs.push_back(xi);
        es.push_back(epsm1);
    }
    std::fclose(f);
    if (!ok || xs.empty()) { std::free(m); return nullptr; }
    m->points = xs.size();
    m->xi = (double *)std::malloc(xs.size() * sizeof(double));
    m->epsm1 = (double *)std::malloc(es.size() * sizeof(double));
    std::memcpy(m->xi, xs.data(), xs.size() * sizeof(double));
    std::memcpy(m->epsm1, es.data(), es.size() * sizeof(double));
    m->xi_min = xs.front();
    m->xi_max = xs.back();
    // the file gives eV; the callbacks work in rad/s
    m->omegap_low /= CAPS_hbar_eV;
    m->omegap_high /= CAPS_hbar_eV;
    m->gamma_low /= CAPS_hbar_eV;
    m->gamma_high /= CAPS_hbar_eV;
    return m;
}

extern "C" void material_free(material_t *m)
{
    if (!m) return;
    std::free(m->xi);
    std::free(m->epsm1);
    std::free(m);
}

extern "C" void material_get_extrapolation(material_t *m, double *omegap_low, double *gamma_low, double *omegap_high,
                                           double *gamma_high)
{
    if (omegap_low) *omegap_low = m->omegap_low;
    if (gamma_low) *gamma_low = m->gamma_low;
    if (omegap_high) *omegap_high = m->omegap_high;
    if (gamma_high) *gamma_high = m->gamma_high;
}

extern "C" void material_info(material_t *m, FILE *stream, const char *prefix)
{
    if (!prefix) prefix = "";
    std::fprintf(stream, "%sfilename    = %s\n", prefix, m->filename);
    std::fprintf(stream, "%spoints      = %zu\n", prefix, m->points);
    std::fprintf(stream, "%scalL        = %gm\n", prefix, m->calL);
    std::fprintf(stream, "%sxi_min      = %g/m\n", prefix, m->xi_min);
    std::fprintf(stream, "%sxi_max      = %g/m\n", prefix, m->xi_max);
    std::fprintf(stream, "%somegap_high = %geV\n", prefix, CAPS_hbar_eV * m->omegap_high);
    std::fprintf(stream, "%sgamma_high  = %geV\n", prefix, CAPS_hbar_eV * m->gamma_high);
    std::fprintf(stream, "%sgamma_low   = %geV\n", prefix, CAPS_hbar_eV * m->gamma_low);
    std::fprintf(stream, "%somegap_low  = %geV\n", prefix, CAPS_hbar_eV * m->omegap_low);
}

// eps(i xi) - 1 for xi in rad/s: Drude outside the table, linear interpolation inside
extern "C" double material_epsilonm1(double xi, void *args)
{
    const material_t *m = (const material_t *)args;
    if (xi < m->xi_min) return m->omegap_low * m->omegap_low / (xi * (xi + m->gamma_low));
    if (xi > m->xi_max) return m->omegap_high * m->omegap_high / (xi * (xi + m->gamma_high));
    if (m->points < 2) return m->epsm1[0];
    // bracketing pair by bisection: xi[lo] <= xi < xi[hi] (hi = lo + 1)
    int lo = 0, hi = (int)m->points - 1;
    while (hi - lo != 1) {
        const int mid = (lo + hi) / 2;
        if (m->xi[mid] > xi) hi = mid; else lo = mid;
    }
    const double x0 = m->xi[lo], x1 = m->xi[hi], e0 = m->epsm1[lo], e1 = m->epsm1[hi];
    return e0 + (xi - x0) * (e1 - e0) / (x1 - x0);
}
