// The reference's text output (include/hfx_report.h), restating
// Util/PrettyPrint.hs:83-211 and the libraries it prints with:
//   numbers   GHC Numeric (base < 4.6, the reference's bytestring < 0.10 era):
//             floatToDigits' shortest round-trip digits (std::to_chars here),
//             roundTo halving up on the first dropped digit, and the
//             FFFixed / FFExponent / FFGeneric layouts of formatRealFloat
//   tables    ppAsRows q: every column padded to its widest cell plus q
//             spaces, cells joined by one space (hsep), rows by newlines
//   details   boxes: "n." right-aligned in 3 columns, two spaces, the
//             header flowed into lines of at most 95 columns; each flowed
//             line keeps one space after its last word, as the reference's
//             own output files show (tests/spectra/*.out), and every line
//             is padded to the widest
// The pretty, boxes and base packages are not in the reference tree; the
// column layout is pinned by those output files.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/hfx_report.h"

namespace {

constexpr float kHostH = 1.007276f;  // Mass.hs:25

// floatToDigits 10 x (x > 0): digits d1 d2 ... (no trailing zeros) and e
// with x = 0.d1d2... * 10^e.
template <typename T>
void float_digits(T x, std::vector<int> &ds, int &e) {
    ds.clear();
    if (x == 0) {
        ds.push_back(0);
        e = 0;
        return;
    }
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::scientific);
    const char *p = buf;
    for (; p < r.ptr && *p != 'e'; ++p)
        if (*p >= '0' && *p <= '9') ds.push_back(*p - '0');
    int ex = 0;
    std::from_chars(p + 1 + (p[1] == '+' ? 1 : 0), r.ptr, ex);
    while (ds.size() > 1 && ds.back() == 0) ds.pop_back();
    e = ex + 1;
}

// roundTo 10 d is: is rounded to d digits, halves up; the carry says
// whether a digit was added in front.
int round_to(int d, const std::vector<int> &is, std::vector<int> &out) {
    out.assign((size_t)(d > 0 ? d : 0), 0);
    int c = (size_t)d < is.size() && d >= 0 ? (is[(size_t)d] >= 5 ? 1 : 0) : 0;
    for (int k = d - 1; k >= 0; --k) {
        const int v = ((size_t)k < is.size() ? is[(size_t)k] : 0) + c;
        out[(size_t)k] = v == 10 ? 0 : v;
        c = v == 10 ? 1 : 0;
    }
    if (c) out.insert(out.begin(), 1);
    return c;
}

std::string digits_str(const std::vector<int> &v, size_t a, size_t b) {
    std::string s;
    for (size_t i = a; i < b && i < v.size(); ++i) s.push_back((char)('0' + v[i]));
    return s;
}

template <typename T>
bool special(T x, std::string &s) {
    if (std::isnan(x)) {
        s = "NaN";
        return true;
    }
    if (std::isinf(x)) {
        s = x < 0 ? "-Infinity" : "Infinity";
        return true;
    }
    return false;
}

// showFFloat (Just dec)
template <typename T>
std::string show_ffloat(T x, int dec) {
    std::string s;
    if (special(x, s)) return s;
    if (x < 0 || (x == 0 && std::signbit(x))) return "-" + show_ffloat<T>(-x, dec);
    std::vector<int> is, r;
    int e;
    float_digits(x, is, e);
    if (e >= 0) {
        const int ei = round_to(dec + e, is, r);
        std::string ls = digits_str(r, 0, (size_t)(e + ei)), rs = digits_str(r, (size_t)(e + ei), r.size());
        if (ls.empty()) ls = "0";
        return rs.empty() ? ls : ls + "." + rs;
    }
    std::vector<int> z((size_t)(-e), 0);
    z.insert(z.end(), is.begin(), is.end());
    const int ei = round_to(dec, z, r);
    if (!ei) r.insert(r.begin(), 0);
    const std::string all = digits_str(r, 0, r.size());
    return all.size() == 1 ? all : all.substr(0, 1) + "." + all.substr(1);
}

// showEFloat (Just dec)
template <typename T>
std::string show_efloat(T x, int dec) {
    std::string s;
    if (special(x, s)) return s;
    if (x < 0 || (x == 0 && std::signbit(x))) return "-" + show_efloat<T>(-x, dec);
    const int d = dec < 1 ? 1 : dec;
    std::vector<int> is, r;
    int e;
    float_digits(x, is, e);
    if (is.size() == 1 && is[0] == 0) return "0." + std::string((size_t)d, '0') + "e0";
    const int ei = round_to(d + 1, is, r);
    if (ei) r.pop_back();
    return digits_str(r, 0, 1) + "." + digits_str(r, 1, r.size()) + "e" + std::to_string(e - 1 + ei);
}

// show (Float): FFGeneric Nothing
std::string show_float(float x) {
    std::string s;
    if (special(x, s)) return s;
    if (x < 0 || (x == 0 && std::signbit(x))) return "-" + show_float(-x);
    std::vector<int> is;
    int e;
    float_digits(x, is, e);
    const std::string ds = digits_str(is, 0, is.size());
    if (e < 0 || e > 7) {
        if (ds == "0") return "0.0e0";
        if (ds.size() == 1) return ds + ".0e" + std::to_string(e - 1);
        return ds.substr(0, 1) + "." + ds.substr(1) + "e" + std::to_string(e - 1);
    }
    if (e == 0) return "0." + ds;
    std::string ls = ds.substr(0, std::min(ds.size(), (size_t)e));
    if (ls.size() < (size_t)e) ls += std::string((size_t)e - ls.size(), '0');
    std::string rs = (size_t)e < ds.size() ? ds.substr((size_t)e) : "";
    return ls + "." + (rs.empty() ? "0" : rs);
}

// ppAsRows q
std::string pp_as_rows(const std::vector<std::vector<std::string>> &rows, int q) {
    size_t nc = 0;
    for (const auto &r : rows) nc = std::max(nc, r.size());
    std::vector<size_t> w(nc, 0);
    for (const auto &r : rows)
        for (size_t c = 0; c < r.size(); ++c) w[c] = std::max(w[c], r[c].size());
    std::string out;
    for (size_t i = 0; i < rows.size(); ++i) {
        if (i) out.push_back('\n');
        for (size_t c = 0; c < nc; ++c) {
            const std::string cell = c < rows[i].size() ? rows[i][c] : std::string();
            if (c) out.push_back(' ');
            out += cell;
            out.append(w[c] - cell.size() + (size_t)q, ' ');
        }
    }
    return out;
}

int64_t emit(const std::string &s, char *out, int64_t cap) {
    if (out && cap > 0) {
        const size_t k = std::min(s.size(), (size_t)(cap - 1));
        std::memcpy(out, s.data(), k);
        out[k] = '\0';
    }
    return (int64_t)s.size();
}

std::string str(const char *s) { return s ? std::string(s) : std::string(); }

std::vector<std::string> words(const std::string &s) {
    std::vector<std::string> w;
    std::string cur;
    for (char ch : s) {
        if (ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r' || ch == '\f' || ch == '\v') {
            if (!cur.empty()) w.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(ch);
        }
    }
    if (!cur.empty()) w.push_back(cur);
    return w;
}

// boxes' para left n: words flowed greedily, a word fitting while the line
// (each word counted with its following space) stays within n
std::vector<std::string> flow(const std::string &text, size_t n) {
    std::vector<std::string> lines;
    std::string line;
    size_t len = 0;
    for (const std::string &w : words(text)) {
        if (len != 0 && len + w.size() + 1 > n) {
            lines.push_back(line);
            line.clear();
            len = 0;
        }
        line += w;
        line.push_back(' ');
        len += w.size() + 1;
    }
    if (len) lines.push_back(line);
    for (auto &l : lines)
        if (l.size() > n) l.resize(n);
    return lines;
}

}  // namespace

extern "C" {

int64_t hfx_format_number(double x, int32_t kind, char *out, int64_t cap) {
    std::string s;
    switch (kind) {
        case 0: s = show_float((float)x); break;
        case 1: s = show_ffloat<float>((float)x, 4); break;
        case 2: s = show_ffloat<double>(x, 4); break;
        case 3: s = show_efloat<double>(x, 4); break;
        default: return -1;
    }
    return emit(s, out, cap);
}

int64_t hfx_format_rows(const char *const *cells, int32_t nrows, int32_t ncols, int32_t q, char *out, int64_t cap) {
    if (nrows < 0 || ncols < 0 || (nrows && ncols && !cells) || q < 0) return -1;
    std::vector<std::vector<std::string>> rows((size_t)nrows);
    for (int32_t i = 0; i < nrows; ++i)
        for (int32_t c = 0; c < ncols; ++c) rows[(size_t)i].push_back(str(cells[(size_t)i * ncols + c]));
    return emit(pp_as_rows(rows, q), out, cap);
}

int64_t hfx_format_results(const hfx_result_row *rows, int32_t n, int32_t all, char *out, int64_t cap) {
    if (n < 0 || (n && !rows)) return -1;
    // PrettyPrint.hs:101-107 title / titleAll
    std::vector<std::vector<std::string>> t = {
        {" # ", " (M+H)+  ", "deltCn", "XCorr", "Ions", "Reference", "Peptide", "E-value"},
        {"---", "---------", "------", "-----", "----", "---------", "-------", "-------"}};
    if (all) {
        t[0].insert(t[0].end(), {"Scan details", "File"});
        t[1].insert(t[1].end(), {"------------", "----"});
    }
    const float s0 = n ? rows[0].xcorr : 0.0f;
    for (int32_t i = 0; i < n; ++i) {
        const hfx_result_row &m = rows[i];
        const float dcn = (s0 - m.xcorr) / s0;  // Float, shown as Double (realToFrac)
        std::vector<std::string> r = {" " + std::to_string(i + 1) + ".",
                                      show_ffloat<float>(m.mh, 4),
                                      show_ffloat<double>((double)dcn, 4),
                                      show_ffloat<double>((double)m.xcorr, 4),
                                      std::to_string(m.ions_matched) + "/" + std::to_string(m.ions_total),
                                      str(m.reference),
                                      str(m.peptide),
                                      show_efloat<double>(m.evalue, 4)};
        if (all) {
            r.push_back(str(m.scan));
            r.push_back(str(m.file));
        }
        t.push_back(r);
    }
    return emit(pp_as_rows(t, 1) + "\n\n", out, cap);
}

int64_t hfx_format_config(const char *title, const char *spectrum, const char *database, const char *enzyme,
                          float pcr, float charge, float tol, char *out, int64_t cap) {
    const float mass = (pcr * charge) - ((charge * kHostH) - 1.0f);
    const long z = std::lrint(charge);  // round: halves to even
    std::string ez;
    for (const std::string &w : words(str(enzyme))) ez += (ez.empty() ? "" : " ") + w;
    const std::string m = show_float(mass) + " ~ " + show_float(tol) + " (" + (z < 0 ? "-" : "+") +
                          std::to_string(z) + ")";
    const std::vector<std::vector<std::string>> rows = {{"Title", "::", str(title)},
                                                        {"Spectrum", "::", str(spectrum)},
                                                        {"Database", "::", str(database)},
                                                        {"Enzyme", "::", ez},
                                                        {"(M+H)+ Mass", "::", m}};
    return emit(pp_as_rows(rows, 0) + "\n\n", out, cap);
}

int64_t hfx_format_detail(const char *const *headers, int32_t n, char *out, int64_t cap) {
    if (n < 0 || (n && !headers)) return -1;
    std::vector<std::string> lines;
    size_t width = 0;
    for (int32_t i = 0; i < n; ++i) {
        std::string num = std::to_string(i + 1) + ".";
        if (num.size() < 3) num = std::string(3 - num.size(), ' ') + num;
        const std::vector<std::string> para = flow(str(headers[i]), 95);
        size_t pw = 0;
        for (const auto &l : para) pw = std::max(pw, l.size());
        const size_t h = std::max<size_t>(1, para.size());
        for (size_t k = 0; k < h; ++k) {
            std::string l = (k == 0 ? num : std::string(num.size(), ' ')) + "  ";
            std::string p = k < para.size() ? para[k] : std::string();
            p.append(pw - p.size(), ' ');
            lines.push_back(l + p);
            width = std::max(width, lines.back().size());
        }
    }
    std::string s;
    for (auto &l : lines) s += l + std::string(width - l.size(), ' ') + "\n";
    return emit(s + "\n", out, cap);
}

}  // extern "C"
