// ks_gfall.cpp -- native reader of gfall line lists.
//
// Follows synthe_py/io/lines/atomic.py:299-611 (load_catalog: fixed-width
// records of >= 98 columns, else the whitespace form), :718-816
// (filter_by_range DELLIM window) and the routing of
// synthe_py/physics/line_opacity.py:740-784 (which records TRANSP processes)
// and :1094 (which records add their centre to ASYNTH).  Lines are parsed in
// parallel over file chunks; the result keeps file order unless sorting by
// wavelength is requested (stable, with the catalog index kept).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/kurucz_gb300.h"

namespace {

// synthe_py/io/lines/tfort.py:14 _ELEMENT_SYMBOLS (Z = 1..92)
const char* kSymbols[] = {
    "",   "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si",
    "P",  "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu",
    "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru",
    "Rh", "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr",
    "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",
    "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po", "At", "Rn", "Fr", "Ra", "Ac",
    "Th", "Pa", "U"};
const int kNSym = 93;
// opacity.py:316-416 _ELEMENT_Z also knows Np..Es (93..99)
const char* kExtraUpper[] = {"NP", "PU", "AM", "CM", "BK", "CF", "ES"};

const double kDellim[7] = {100.0, 30.0, 10.0, 3.0, 1.0, 0.3, 0.1};

struct Rec {
    double wl, loggf, code, elo, gr, gs, gw;
    int nelem, ion, lt, nblo, nbup, line_size, anum, iso1, iso2;
    double grl, gsl, gwl;  // the GR / GS / GW fields as read (log10; 0 when blank)
    double xj, xjp;        // J of the lower / upper level (columns 37-41, 65-69; 0 when blank)
    bool continuum_label;  // LABELP begins with CONTINUU (a merged-continuum record)
    bool is_h_elem;  // element symbol is H / D (DELLIM special case)
};

// Python str.strip() of a fixed-width field, then float(); false on error.
bool field_float(const char* line, int len, int a, int b, double* out, bool* empty) {
    if (a >= len) {
        *empty = true;
        return true;
    }
    if (b > len) b = len;
    while (a < b && std::isspace((unsigned char)line[a])) a++;
    while (b > a && std::isspace((unsigned char)line[b - 1])) b--;
    if (a == b) {
        *empty = true;
        return true;
    }
    *empty = false;
    char buf[64];
    int n = b - a;
    if (n >= 63) return false;
    std::memcpy(buf, line + a, n);
    buf[n] = 0;
    char* end = nullptr;
    double v = std::strtod(buf, &end);
    if (end != buf + n) return false;
    *out = v;
    return true;
}

bool field_int(const char* line, int len, int a, int b, int* out, bool* empty) {
    double v;
    if (!field_float(line, len, a, b, &v, empty)) return false;
    if (*empty) return true;
    // int("…") in Python rejects decimals; accept only integral text
    for (int i = a; i < std::min(b, len); i++) {
        char ch = line[i];
        if (ch == '.' || ch == 'e' || ch == 'E') return false;
    }
    *out = (int)v;
    return true;
}

int symbol_to_z(const std::string& sym) {
    std::string u;
    for (char ch : sym)
        if (!std::isspace((unsigned char)ch)) u += (char)std::toupper((unsigned char)ch);
    for (int z = 1; z < kNSym; z++) {
        std::string s = kSymbols[z];
        for (auto& ch : s) ch = (char)std::toupper((unsigned char)ch);
        if (s == u) return z;
    }
    for (int i = 0; i < 7; i++)
        if (u == kExtraUpper[i]) return 93 + i;
    return 0;
}

int potion_index(int iz, int icharge) {
    int idx = iz <= 30 ? iz * (iz + 1) / 2 + icharge : iz * 5 + 341 + icharge;
    return idx - 1;
}

// atomic.py:59-106
double stark_default(double code, double elo, double eup, const double* potion, int np) {
    if (code >= 100.0) return -5.0;
    int nelem = (int)(code + 1e-6);
    int icharge = (int)((code - nelem) * 100.0 + 0.1);
    int zeff = icharge + 1;
    double effnsq = 25.0;
    int index = potion_index(nelem, icharge);
    if (potion && index >= 0 && index < np) {
        double deleup = potion[index] - eup;
        if (deleup > 0) effnsq = 109737.31 * zeff * zeff / deleup;
    }
    return std::log10(1.0e-8 * effnsq * effnsq * std::sqrt(effnsq));
}

// atomic.py:109-199
double vdw_default(double code, double elo, double eup, const double* potion, int np) {
    int nelem = (int)(code + 1e-6);
    int icharge = (int)((code - nelem) * 100.0 + 0.1);
    int zeff = icharge + 1;
    if (code >= 100.0) return std::log10(1.0e-7 / zeff);
    int index = potion_index(nelem, icharge);
    double ip = (potion && index >= 0 && index < np) ? potion[index] : 0.0;
    double eu = 25.0;
    if (ip > 0 && ip - eup > 0) eu = 109737.31 * zeff * zeff / (ip - eup);
    eu = std::min(eu, 1000.0);
    double rsqup = 2.5 * (eu / zeff) * (eu / zeff);
    double el = 25.0;
    if (ip > 0 && ip - elo > 0) el = 109737.31 * zeff * zeff / (ip - elo);
    el = std::min(el, 1000.0);
    double rsqlo = 2.5 * (el / zeff) * (el / zeff);
    int nseq = nelem - zeff + 1;
    if (20 < nseq && nseq < 29) {
        rsqup = (45.0 - nseq) / zeff;
        rsqlo = 0.0;
    }
    if (rsqup < rsqlo) rsqup = 2.0 * rsqlo;
    double diff = rsqup - rsqlo;
    double gammaw = diff > 0 ? 4.5e-9 * std::pow(diff, 0.4) : 1.0e-9;
    return std::log10(gammaw);
}

// Python round() (half to even) of frac*100
int py_round(double x) { return (int)std::nearbyint(x); }

bool parse_fixed(const char* line, int len, const double* potion, int np, Rec* r) {
    double wl, loggf_raw, code, e_val, ep_val = 0.0, grl = 0.0, gsl = 0.0, gwl = 0.0;
    bool em;
    if (!field_float(line, len, 0, 11, &wl, &em) || em) return false;
    if (!field_float(line, len, 11, 18, &loggf_raw, &em) || em) return false;
    if (!field_float(line, len, 18, 24, &code, &em) || em) return false;
    if (!field_float(line, len, 24, 36, &e_val, &em) || em) return false;
    if (!field_float(line, len, 52, 64, &ep_val, &em)) return false;
    if (em) ep_val = 0.0;
    if (!field_float(line, len, 80, 86, &grl, &em)) return false;
    if (em) grl = 0.0;
    if (!field_float(line, len, 86, 92, &gsl, &em)) return false;
    if (em) gsl = 0.0;
    if (!field_float(line, len, 92, 98, &gwl, &em)) return false;
    if (em) gwl = 0.0;
    double xj = 0.0, xjp = 0.0;
    if (!field_float(line, len, 36, 41, &xj, &em)) return false;
    if (em) xj = 0.0;
    if (!field_float(line, len, 64, 69, &xjp, &em)) return false;
    if (em) xjp = 0.0;
    bool cont_label = false;
    if (len >= 78) {
        // LABELP (columns 71-78), stripped and upper-cased, starts with CONTINUU
        int a0 = 70, a1 = 78;
        while (a0 < a1 && std::isspace((unsigned char)line[a0])) a0++;
        const char* key = "CONTINUU";
        cont_label = a1 - a0 >= 8;
        for (int k = 0; cont_label && k < 8; k++)
            if (std::toupper((unsigned char)line[a0 + k]) != key[k]) cont_label = false;
    }
    double x1 = 0.0, x2 = 0.0, v;
    if (len >= 115 && field_float(line, len, 109, 115, &v, &em) && !em) x1 = v;
    if (len >= 124 && field_float(line, len, 118, 124, &v, &em) && !em) x2 = v;
    double log_gf = loggf_raw + (x1 + x2);
    double elo = std::min(std::fabs(e_val), std::fabs(ep_val));
    double eup = std::max(std::fabs(e_val), std::fabs(ep_val));
    double gr = grl == 0.0 ? 0.0 : std::pow(10.0, grl);
    double gs = gsl == 0.0 ? 0.0 : std::pow(10.0, gsl);
    double gw = gwl == 0.0 ? 0.0 : std::pow(10.0, gwl);
    double wavelength = wl;
    double eshift = 0.0, eshiftp = 0.0;
    if (len >= 134) {
        bool blank = true;
        for (int i = 124; i < 134; i++)
            if (!std::isspace((unsigned char)line[i])) blank = false;
        if (!blank) {
            int a = 0, b = 0;
            bool e1, e2;
            if (field_int(line, len, 124, 129, &a, &e1) && field_int(line, len, 129, 134, &b, &e2) &&
                !e1 && !e2) {
                eshift = a * 1.0e-3;
                eshiftp = b * 1.0e-3;
            }
        }
    }
    double ediff = std::fabs((std::fabs(ep_val) + eshiftp) - (std::fabs(e_val) + eshift));
    if (ediff > 0.0) {
        double dwliso = 0.0;
        int iso = 0;
        bool e3;
        if (len >= 160 && field_int(line, len, 154, 160, &iso, &e3) && !e3) dwliso = iso * 1.0e-4;
        wavelength = 1.0e7 / ediff + dwliso;
    }
    if (gr == 0.0) gr = 2.223e13 / (wavelength * wavelength);
    if (gs == 0.0) {
        double lv = stark_default(code, elo, eup, potion, np);
        gs = lv != 0.0 ? std::pow(10.0, lv) : 0.0;
    }
    if (gw == 0.0) {
        double lv = vdw_default(code, elo, eup, potion, np);
        gw = lv != 0.0 ? std::pow(10.0, lv) : 0.0;
    }
    double frelin = 2.99792458e17 / std::max(wavelength, 1e-12);
    gr = gr / (12.5664 * frelin);
    gs = gs / (12.5664 * frelin);
    gw = gw / (12.5664 * frelin);
    int nelem = (int)(code + 1e-6);
    double frac = code - nelem;
    int ion = frac > 1e-6 ? py_round(frac * 100.0) + 1 : 1;
    int nblo = 0, nbup = 0;
    if (len >= 106) {
        int a = 0, b = 0;
        bool e1, e2;
        if (field_int(line, len, 102, 104, &a, &e1) && field_int(line, len, 104, 106, &b, &e2)) {
            nblo = e1 ? 0 : a;
            nbup = e2 ? 0 : b;
        }
    }
    int iso1 = 0;
    if (len >= 109) {
        int a;
        bool e1;
        if (field_int(line, len, 106, 109, &a, &e1) && !e1) iso1 = a;
    }
    int iso2 = 0;
    if (len >= 119) {
        int a;
        bool e1;
        if (field_int(line, len, 116, 119, &a, &e1) && !e1) iso2 = a;
    }
    int line_size = 0;
    std::string tag;
    if (len >= 144) {
        bool blank = true;
        for (int i = 134; i < 144; i++)
            if (!std::isspace((unsigned char)line[i])) blank = false;
        if (!blank) {
            char ls = line[140];
            for (int i = 141; i < 144; i++)
                if (!std::isspace((unsigned char)line[i])) tag += line[i];
            if (ls >= '0' && ls <= '9') line_size = ls - '0';
        }
    }
    int lt = 0;
    if (tag == "AUT") lt = 1;
    else if (tag == "COR") lt = 2;
    else if (tag == "PRD") lt = 3;
    else if (nelem == 1 && ion == 1 && iso1 == 2) lt = -2;
    else if (nelem == 1 && ion == 1) lt = -1;
    else if (nelem == 2 && ion == 1 && iso1 == 3) lt = -4;
    else if (nelem == 2 && ion == 1) lt = -3;
    else if (nelem == 2 && ion == 2) lt = -6;
    r->wl = wavelength;
    r->loggf = log_gf;
    r->code = code;
    r->elo = elo;
    r->gr = gr;
    r->gs = gs;
    r->gw = gw;
    r->nelem = nelem;
    r->ion = ion;
    r->lt = lt;
    r->nblo = nblo;
    r->nbup = nbup;
    r->line_size = line_size;
    r->iso1 = iso1;
    r->iso2 = iso2;
    r->grl = grl;
    r->gsl = gsl;
    r->gwl = gwl;
    r->xj = xj;
    r->xjp = xjp;
    r->continuum_label = cont_label;
    // element symbol: tfort symbols up to U, else "Z<n>" (unknown to TRANSP)
    r->anum = (nelem > 0 && nelem < kNSym) ? nelem : 0;
    r->is_h_elem = nelem == 1;
    return true;
}

// atomic.py:617-682 whitespace form: wl element ion loggf E gr gs [gw [nlo nup]]
bool parse_ws(const char* line, int len, Rec* r) {
    std::vector<std::string> parts;
    std::string cur;
    for (int i = 0; i < len; i++) {
        if (std::isspace((unsigned char)line[i])) {
            if (!cur.empty()) parts.push_back(cur), cur.clear();
        } else {
            cur += line[i];
        }
    }
    if (!cur.empty()) parts.push_back(cur);
    if (parts.size() < 7) return false;
    auto num = [](const std::string& s, double* v) {
        char* end = nullptr;
        *v = std::strtod(s.c_str(), &end);
        return end == s.c_str() + s.size();
    };
    double wl, ionf, loggf, exc, gr, gs, gw = 0.0;
    if (!num(parts[0], &wl) || !num(parts[2], &ionf) || !num(parts[3], &loggf) ||
        !num(parts[4], &exc) || !num(parts[5], &gr) || !num(parts[6], &gs))
        return false;
    if (parts.size() > 7 && !num(parts[7], &gw)) return false;
    int nlo = 0, nup = 0;
    if (parts.size() > 9) {
        double a, b;
        if (num(parts[8], &a) && num(parts[9], &b)) {
            nlo = (int)a;
            nup = (int)b;
        }
    }
    const std::string& el = parts[1];
    int ion = (int)ionf;
    int lt = 0;
    if (el == "H" && ion == 1) lt = -1;
    else if (el == "He" && ion == 1) lt = -3;
    else if (el == "He" && ion == 2) lt = -6;
    int z = symbol_to_z(el);
    r->wl = wl;
    r->loggf = loggf;
    r->code = 0.0;
    r->elo = exc;
    r->gr = gr;
    r->gs = gs;
    r->gw = gw;
    r->nelem = z;
    r->ion = ion;
    r->lt = lt;
    r->nblo = nlo;
    r->nbup = nup;
    r->line_size = 0;
    r->iso1 = 0;
    r->iso2 = 0;
    r->grl = r->gsl = r->gwl = 0.0;
    r->xj = r->xjp = 0.0;
    r->continuum_label = false;
    r->anum = z;
    std::string u;
    for (char ch : el) u += (char)std::toupper((unsigned char)ch);
    r->is_h_elem = (el == "H" || el == "D");
    (void)u;
    return true;
}

}  // namespace

struct ks_gfall {
    std::vector<Rec> recs;
    std::vector<int64_t> index;  // catalog position of each output row
};

extern "C" ks_status ks_gfall_read(const char* path, double wl_min, double wl_max,
                                   const double* potion, int32_t n_potion, ks_gfall** out) {
    if (!path || !out) return KS_ERR_INVALID;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return KS_ERR_IO;
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::string text(sz > 0 ? (size_t)sz : 0, '\0');
    if (sz > 0 && std::fread(&text[0], 1, (size_t)sz, f) != (size_t)sz) {
        std::fclose(f);
        return KS_ERR_IO;
    }
    std::fclose(f);
    // line starts (splitlines on \n, \r\n or \r)
    std::vector<size_t> starts, lens;
    size_t i = 0, n = text.size();
    while (i < n) {
        size_t j = i;
        while (j < n && text[j] != '\n' && text[j] != '\r') j++;
        starts.push_back(i);
        lens.push_back(j - i);
        if (j < n && text[j] == '\r' && j + 1 < n && text[j + 1] == '\n') j++;
        i = j + 1;
    }
    size_t nl = starts.size();
    std::vector<Rec> recs(nl);
    std::vector<char> ok(nl, 0);
    unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; t++) {
        th.emplace_back([&, t]() {
            for (size_t k = t; k < nl; k += nth) {
                const char* line = text.data() + starts[k];
                int len = (int)lens[k];
                int a = 0, b = len;
                while (a < b && std::isspace((unsigned char)line[a])) a++;
                while (b > a && std::isspace((unsigned char)line[b - 1])) b--;
                if (a == b || line[a] == '#') continue;
                if (len >= 98 && parse_fixed(line, len, potion, n_potion, &recs[k])) ok[k] = 1;
                else if (len < 98 && parse_ws(line, len, &recs[k])) ok[k] = 1;
            }
        });
    }
    for (auto& x : th) x.join();
    ks_gfall* g = new ks_gfall();
    double delfactor = wl_min <= 500.0 ? 1.0 : wl_min / 500.0;
    for (size_t k = 0; k < nl; k++) {
        if (!ok[k]) continue;
        const Rec& r = recs[k];
        if (wl_max > 0.0) {
            int lim = std::min(8 - (r.line_size > 0 ? r.line_size : 0), 7);
            if (std::fabs(r.code - 1.0) < 1.0e-6 || r.lt == -1 || r.lt == -2 || r.is_h_elem) lim = 1;
            lim = std::max(1, std::min(7, lim));
            double margin = kDellim[lim - 1] * delfactor;
            if (!(r.wl >= wl_min - margin && r.wl <= wl_max + margin)) continue;
        }
        g->recs.push_back(r);
    }
    g->index.resize(g->recs.size());
    std::iota(g->index.begin(), g->index.end(), 0);
    *out = g;
    return KS_OK;
}

extern "C" int64_t ks_gfall_count(const ks_gfall* g) { return g ? (int64_t)g->recs.size() : -1; }

extern "C" ks_status ks_gfall_sort(ks_gfall* g) {
    if (!g) return KS_ERR_INVALID;
    std::vector<int64_t> order(g->recs.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t a, int64_t b) { return g->recs[a].wl < g->recs[b].wl; });
    std::vector<Rec> r2(order.size());
    std::vector<int64_t> i2(order.size());
    for (size_t k = 0; k < order.size(); k++) {
        r2[k] = g->recs[order[k]];
        i2[k] = g->index[order[k]];
    }
    g->recs.swap(r2);
    g->index.swap(i2);
    return KS_OK;
}

extern "C" ks_status ks_gfall_fetch(const ks_gfall* g, double* wavelength, double* log_gf, double* gf,
                                    double* cgf, double* elo_cm, double* gamma_rad,
                                    double* gamma_stark, double* gamma_vdw, int32_t* element_idx,
                                    int32_t* ion_stage, int32_t* line_type, uint8_t* process_mask,
                                    uint8_t* asynth_mask, double* code, int64_t* catalog_index) {
    if (!g) return KS_ERR_INVALID;
    const double cgf_const = 0.026538 / 1.77245;
    for (size_t k = 0; k < g->recs.size(); k++) {
        const Rec& r = g->recs[k];
        double gfv = std::pow(10.0, r.loggf);
        if (wavelength) wavelength[k] = r.wl;
        if (log_gf) log_gf[k] = r.loggf;
        if (gf) gf[k] = gfv;
        if (cgf) cgf[k] = cgf_const * gfv / (2.99792458e17 / r.wl);
        if (elo_cm) elo_cm[k] = r.elo;
        if (gamma_rad) gamma_rad[k] = r.gr;
        if (gamma_stark) gamma_stark[k] = r.gs;
        if (gamma_vdw) gamma_vdw[k] = r.gw;
        int anum = r.anum;
        if (element_idx) element_idx[k] = anum > 0 ? anum - 1 : -1;
        if (ion_stage) ion_stage[k] = r.ion;
        if (line_type) line_type[k] = r.lt;
        bool fort12 = r.lt != 2 && r.lt != 1 && r.lt <= 3 && (std::abs(r.nblo) + std::abs(r.nbup)) == 0;
        bool is_h = r.is_h_elem && r.ion == 1;
        if (process_mask) process_mask[k] = (fort12 && !(r.lt == -1 || is_h) && anum > 0) ? 1 : 0;
        if (asynth_mask) {
            int t = r.lt;
            asynth_mask[k] = !(t == -2 || t == -1 || t == 1 || t == 2 || t == 3 || t == 4);
        }
        if (code) code[k] = r.code;
        if (catalog_index) catalog_index[k] = g->index[k];
    }
    return KS_OK;
}

extern "C" ks_status ks_gfall_fetch_levels(const ks_gfall* g, int32_t* n_lower, int32_t* n_upper) {
    if (!g) return KS_ERR_INVALID;
    for (size_t k = 0; k < g->recs.size(); k++) {
        if (n_lower) n_lower[k] = g->recs[k].nblo;
        if (n_upper) n_upper[k] = g->recs[k].nbup;
    }
    return KS_OK;
}

extern "C" ks_status ks_gfall_fetch_iso(const ks_gfall* g, int32_t* iso1, int32_t* iso2) {
    if (!g) return KS_ERR_INVALID;
    for (size_t k = 0; k < g->recs.size(); k++) {
        if (iso1) iso1[k] = g->recs[k].iso1;
        if (iso2) iso2[k] = g->recs[k].iso2;
    }
    return KS_OK;
}

extern "C" ks_status ks_gfall_fetch_gamma_logs(const ks_gfall* g, double* gr, double* gs, double* gw) {
    if (!g) return KS_ERR_INVALID;
    for (size_t k = 0; k < g->recs.size(); k++) {
        if (gr) gr[k] = g->recs[k].grl;
        if (gs) gs[k] = g->recs[k].gsl;
        if (gw) gw[k] = g->recs[k].gwl;
    }
    return KS_OK;
}

extern "C" ks_status ks_gfall_fetch_j(const ks_gfall* g, double* xj, double* xjp, uint8_t* continuum_label) {
    if (!g) return KS_ERR_INVALID;
    for (size_t k = 0; k < g->recs.size(); k++) {
        if (xj) xj[k] = g->recs[k].xj;
        if (xjp) xjp[k] = g->recs[k].xjp;
        if (continuum_label) continuum_label[k] = g->recs[k].continuum_label ? 1 : 0;
    }
    return KS_OK;
}

extern "C" void ks_gfall_free(ks_gfall* g) { delete g; }
