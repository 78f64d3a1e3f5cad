// Input formats on both sides of the search (include/hfx_io.h): MGF and DTA
// spectra, FASTA proteins (plain or gzip) and the digested-database .index
// file.  Host code only.
//
// The grammars follow the reference's parsers line by line:
//   Util/Parsec.hs:25-85   float tokens (digits, '.', '-') after spaces/tabs,
//                          read with readSigned readFloat (the first number
//                          lexeme; a token with no number is an error),
//                          key = value parameters (value up to '#' or the
//                          line end, trailing white space removed), eol = one
//                          or more '\n'/'\r'
//   Spectrum/MGF.hs:48-75  BEGIN IONS, parameters, "mz intensity" lines,
//                          END IONS; TITLE, CHARGE, PEPMASS (first of each);
//                          a zero or missing charge or mass is an error
//   Spectrum/DTA.hs:35-55  "mz intensity" lines; the first holds (M+H)+ and an
//                          integral charge, pcr = (m + (c-1) H) / c
//   Sequence/Fasta.hs:27-36 over the bio package's FASTA reader (bio 0.5, not
//                          in the reference tree; its published reader is
//                          restated: non-empty lines, a record per '>' line,
//                          the record's sequence lines up to the first that
//                          does not start with a letter)
//   Sequence/Index.hs:40-82 the options text as a serialised lazy ByteString,
//                          then gzip of the SequenceDB (Fragment.hs:165-172)
//                          serialised by the binary package (binary 0.5,
//                          vector-binary-instances 0.1, not in the tree; their
//                          published encodings are restated: Int as big-endian
//                          Int64, Word32 big-endian, a vector as its length
//                          then its elements, a Float as decodeFloat's
//                          (Integer mantissa, Int exponent), an Integer as
//                          tag 0 + Int32 or tag 1 + sign + little-endian bytes)
// gzip (RFC 1952) and deflate (RFC 1951) are decoded here, from the RFCs,
// so the library needs no zlib.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/hfx_io.h"

namespace {

constexpr float kHostH = 1.007276f;  // Mass.hs:25

struct Fail {
    std::string msg;
};

int32_t report(const Fail &f, char *err, int32_t errcap) {
    if (err && errcap > 0) {
        std::snprintf(err, (size_t)errcap, "%s", f.msg.c_str());
    }
    return 1;  // HFX_ERR_ARG
}

std::vector<uint8_t> read_file(const char *path) {
    std::vector<uint8_t> d;
    FILE *fp = path ? std::fopen(path, "rb") : nullptr;
    if (!fp) throw Fail{std::string("cannot open ") + (path ? path : "(null)")};
    uint8_t buf[1 << 16];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof buf, fp)) > 0) d.insert(d.end(), buf, buf + k);
    const bool bad = std::ferror(fp) != 0;
    std::fclose(fp);
    if (bad) throw Fail{std::string("cannot read ") + path};
    return d;
}

bool ends_with_ci(const std::string &s, const char *suffix) {
    const size_t n = std::strlen(suffix);
    if (s.size() < n) return false;
    for (size_t i = 0; i < n; ++i) {
        char a = s[s.size() - n + i];
        if (a >= 'A' && a <= 'Z') a = (char)(a - 'A' + 'a');
        if (a != suffix[i]) return false;
    }
    return true;
}

// ---------------------------------------------------------------- inflate

uint32_t crc32_of(const uint8_t *p, size_t n, uint32_t crc = 0) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        init = true;
    }
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 255u] ^ (crc >> 8);
    return ~crc;
}

// Canonical Huffman code: counts per length and symbols in code order.
struct Huffman {
    uint16_t count[16];
    std::vector<uint16_t> symbol;
};

void build_huffman(Huffman &h, const uint8_t *lengths, int n) {
    std::memset(h.count, 0, sizeof h.count);
    for (int i = 0; i < n; ++i) h.count[lengths[i]]++;
    h.count[0] = 0;
    int left = 1;
    for (int len = 1; len < 16; ++len) {
        left = (left << 1) - h.count[len];
        if (left < 0) throw Fail{"gzip: over-subscribed Huffman code"};
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int len = 1; len < 15; ++len) offs[len + 1] = (uint16_t)(offs[len] + h.count[len]);
    h.symbol.assign((size_t)n, 0);
    for (int i = 0; i < n; ++i)
        if (lengths[i]) h.symbol[offs[lengths[i]]++] = (uint16_t)i;
}

struct BitReader {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    uint32_t bits(int need) {
        uint32_t v = bitbuf;
        while (bitcnt < need) {
            if (pos >= n) throw Fail{"gzip: truncated data"};
            v |= (uint32_t)p[pos++] << bitcnt;
            bitcnt += 8;
        }
        bitbuf = need < 32 ? v >> need : 0u;
        bitcnt -= need;
        return need < 32 ? v & ((1u << need) - 1u) : v;
    }
    int decode(const Huffman &h) {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= (int)bits(1);
            const int cnt = h.count[len];
            if (code - cnt < first) return h.symbol[(size_t)(index + (code - first))];
            index += cnt;
            first = (first + cnt) << 1;
            code <<= 1;
        }
        throw Fail{"gzip: bad Huffman code"};
    }
    void align() {
        bitbuf = 0;
        bitcnt = 0;
    }
};

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_codes(BitReader &br, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out) {
    while (true) {
        const int sym = br.decode(lit);
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return;
        } else {
            const int li = sym - 257;
            if (li >= 29) throw Fail{"gzip: bad length symbol"};
            const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
            const int di = br.decode(dist);
            if (di >= 30) throw Fail{"gzip: bad distance symbol"};
            const size_t d = kDistBase[di] + br.bits(kDistExtra[di]);
            if (d > out.size()) throw Fail{"gzip: distance before the start"};
            const size_t from = out.size() - d;
            for (size_t i = 0; i < len; ++i) {
                const uint8_t byte = out[from + i];
                out.push_back(byte);
            }
        }
    }
}

// RFC 1951: every block of one deflate stream; returns the bytes consumed.
size_t inflate_stream(const uint8_t *p, size_t n, std::vector<uint8_t> &out) {
    BitReader br{p, n};
    bool last = false;
    while (!last) {
        last = br.bits(1) != 0u;
        const uint32_t type = br.bits(2);
        if (type == 0) {
            br.align();
            if (br.pos + 4 > n) throw Fail{"gzip: truncated stored block"};
            const uint32_t len = (uint32_t)p[br.pos] | ((uint32_t)p[br.pos + 1] << 8);
            const uint32_t nlen = (uint32_t)p[br.pos + 2] | ((uint32_t)p[br.pos + 3] << 8);
            if ((len ^ 0xFFFFu) != nlen) throw Fail{"gzip: stored block length check"};
            br.pos += 4;
            if (br.pos + len > n) throw Fail{"gzip: truncated stored block"};
            out.insert(out.end(), p + br.pos, p + br.pos + len);
            br.pos += len;
        } else if (type == 1) {
            uint8_t l[288 + 30];
            for (int i = 0; i < 144; ++i) l[i] = 8;
            for (int i = 144; i < 256; ++i) l[i] = 9;
            for (int i = 256; i < 280; ++i) l[i] = 7;
            for (int i = 280; i < 288; ++i) l[i] = 8;
            for (int i = 0; i < 30; ++i) l[288 + i] = 5;
            Huffman lit, dist;
            build_huffman(lit, l, 288);
            build_huffman(dist, l + 288, 30);
            inflate_codes(br, lit, dist, out);
        } else if (type == 2) {
            const int nlen = (int)br.bits(5) + 257, ndist = (int)br.bits(5) + 1, ncode = (int)br.bits(4) + 4;
            if (nlen > 286 || ndist > 30) throw Fail{"gzip: bad code counts"};
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < ncode; ++i) cl[order[i]] = (uint8_t)br.bits(3);
            Huffman lencode;
            build_huffman(lencode, cl, 19);
            uint8_t lengths[286 + 30] = {0};
            int i = 0;
            while (i < nlen + ndist) {
                const int sym = br.decode(lencode);
                if (sym < 16) {
                    lengths[i++] = (uint8_t)sym;
                } else {
                    uint8_t v = 0;
                    int rep;
                    if (sym == 16) {
                        if (i == 0) throw Fail{"gzip: repeat with no previous length"};
                        v = lengths[i - 1];
                        rep = 3 + (int)br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.bits(3);
                    } else {
                        rep = 11 + (int)br.bits(7);
                    }
                    if (i + rep > nlen + ndist) throw Fail{"gzip: too many lengths"};
                    while (rep--) lengths[i++] = v;
                }
            }
            if (lengths[256] == 0) throw Fail{"gzip: no end-of-block code"};
            Huffman lit, dist;
            build_huffman(lit, lengths, nlen);
            build_huffman(dist, lengths + nlen, ndist);
            inflate_codes(br, lit, dist, out);
        } else {
            throw Fail{"gzip: bad block type"};
        }
    }
    return br.pos;
}

// RFC 1952: every member of a gzip file, concatenated.
std::vector<uint8_t> gunzip(const uint8_t *p, size_t n) {
    std::vector<uint8_t> out;
    size_t pos = 0;
    while (pos < n) {
        if (n - pos < 18 || p[pos] != 0x1f || p[pos + 1] != 0x8b || p[pos + 2] != 8)
            throw Fail{"not a gzip stream"};
        const uint8_t flg = p[pos + 3];
        size_t q = pos + 10;
        if (flg & 4) {
            if (q + 2 > n) throw Fail{"gzip: truncated header"};
            q += 2 + ((size_t)p[q] | ((size_t)p[q + 1] << 8));
        }
        for (int f = 8; f <= 16; f <<= 1)
            if (flg & f) {
                while (q < n && p[q] != 0) ++q;
                ++q;
            }
        if (flg & 2) q += 2;
        if (q > n) throw Fail{"gzip: truncated header"};
        const size_t start = out.size();
        q += inflate_stream(p + q, n - q, out);
        if (q + 8 > n) throw Fail{"gzip: truncated trailer"};
        const uint32_t crc = (uint32_t)p[q] | ((uint32_t)p[q + 1] << 8) | ((uint32_t)p[q + 2] << 16) |
                             ((uint32_t)p[q + 3] << 24);
        const uint32_t isize = (uint32_t)p[q + 4] | ((uint32_t)p[q + 5] << 8) | ((uint32_t)p[q + 6] << 16) |
                               ((uint32_t)p[q + 7] << 24);
        if (crc32_of(out.data() + start, out.size() - start) != crc) throw Fail{"gzip: CRC mismatch"};
        if ((uint32_t)(out.size() - start) != isize) throw Fail{"gzip: size mismatch"};
        pos = q + 8;
    }
    return out;
}

// gzip with stored deflate blocks.
std::vector<uint8_t> gzip_stored(const std::vector<uint8_t> &d) {
    std::vector<uint8_t> o = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 0xff};
    size_t pos = 0;
    do {
        const size_t len = std::min<size_t>(65535, d.size() - pos);
        const bool last = pos + len == d.size();
        o.push_back(last ? 1 : 0);
        o.push_back((uint8_t)(len & 255));
        o.push_back((uint8_t)(len >> 8));
        o.push_back((uint8_t)(~len & 255));
        o.push_back((uint8_t)((~len >> 8) & 255));
        o.insert(o.end(), d.begin() + (long)pos, d.begin() + (long)(pos + len));
        pos += len;
    } while (pos < d.size());
    const uint32_t crc = crc32_of(d.data(), d.size()), sz = (uint32_t)d.size();
    for (int k = 0; k < 4; ++k) o.push_back((uint8_t)(crc >> (8 * k)));
    for (int k = 0; k < 4; ++k) o.push_back((uint8_t)(sz >> (8 * k)));
    return o;
}

// ---------------------------------------------------------------- numbers

bool is_space(uint8_t c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }
bool is_digit(uint8_t c) { return c >= '0' && c <= '9'; }
bool is_alpha(uint8_t c) { return (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z'); }

// readSigned readFloat, first parse (Numeric): white space, an optional '-'
// lexeme, then a decimal number lexeme (digits, optionally '.' digits,
// optionally e[+-]digits); the value is the lexeme correctly rounded to
// Float.  Returns false when the string does not start with a number.
bool read_signed_float(const char *s, size_t n, float &out) {
    size_t i = 0;
    while (i < n && is_space((uint8_t)s[i])) ++i;
    bool neg = false;
    if (i < n && s[i] == '-') {
        neg = true;
        ++i;
        while (i < n && is_space((uint8_t)s[i])) ++i;
    }
    const size_t a = i;
    while (i < n && is_digit((uint8_t)s[i])) ++i;
    if (i == a) return false;
    if (i + 1 < n && s[i] == '.' && is_digit((uint8_t)s[i + 1])) {
        i += 1;
        while (i < n && is_digit((uint8_t)s[i])) ++i;
    }
    if (i < n && (s[i] == 'e' || s[i] == 'E')) {
        size_t j = i + 1;
        if (j < n && (s[j] == '+' || s[j] == '-')) ++j;
        if (j < n && is_digit((uint8_t)s[j])) {
            while (j < n && is_digit((uint8_t)s[j])) ++j;
            i = j;
        }
    }
    const std::string lexeme(s + a, i - a);
    const float v = std::strtof(lexeme.c_str(), nullptr);
    out = neg ? -v : v;
    return true;
}

// ---------------------------------------------------------------- spectra

struct Text {
    const char *p;
    size_t n, pos = 0;
    size_t line() const {
        size_t l = 1;
        for (size_t i = 0; i < pos && i < n; ++i) l += p[i] == '\n';
        return l;
    }
    [[noreturn]] void fail(const std::string &what) const {
        throw Fail{"line " + std::to_string(line()) + ": " + what};
    }
    bool eof() const { return pos >= n; }
    // eol: one or more '\n' / '\r'
    bool eol() {
        const size_t a = pos;
        while (pos < n && (p[pos] == '\n' || p[pos] == '\r')) ++pos;
        return pos > a;
    }
    // float: spaces/tabs, then one or more of digit . -; 0 = no token and
    // nothing consumed, 1 = token, -1 = spaces consumed but no token
    int token(std::string &t) {
        const size_t a = pos;
        while (pos < n && (p[pos] == ' ' || p[pos] == '\t')) ++pos;
        const size_t b = pos;
        while (pos < n && (is_digit((uint8_t)p[pos]) || p[pos] == '.' || p[pos] == '-')) ++pos;
        if (pos == b) return pos == a ? 0 : -1;
        t.assign(p + b, pos - b);
        return 1;
    }
    // readF2 under endBy ... eol: 1 = a pair, 0 = no pair (nothing consumed)
    int pair(float &x, float &y) {
        std::string t;
        const int r = token(t);
        if (r == 0) return 0;
        if (r < 0) fail("expecting a floating-point number");
        if (!read_signed_float(t.data(), t.size(), x)) fail("no parse of \"" + t + "\"");
        if (token(t) <= 0) fail("expecting a floating-point number");
        if (!read_signed_float(t.data(), t.size(), y)) fail("no parse of \"" + t + "\"");
        if (!eol()) fail("expecting end of line");
        return 1;
    }
    bool lit(const char *s) {
        const size_t k = std::strlen(s);
        if (n - pos < k || std::memcmp(p + pos, s, k) != 0) return false;
        pos += k;
        return true;
    }
};

}  // namespace

struct hfx_spectra {
    std::vector<float> mz, it, pcr, z;
    std::vector<int64_t> off{0};
    std::vector<std::string> title;
};

struct hfx_proteins {
    std::vector<uint8_t> seq;
    std::vector<uint32_t> seg{0};
    std::vector<std::string> header;
};

struct hfx_index {
    std::string options;
    std::vector<std::string> header;
    std::vector<uint8_t> ions;
    std::vector<uint32_t> ion_seg, c, n, frag_seg;
    std::vector<float> r;
};

namespace {

// MGF.hs:48-62 sample, repeated to the end of the text.
void parse_mgf(Text &t, hfx_spectra &s) {
    while (!t.eof()) {
        if (!t.lit("BEGIN IONS")) t.fail("expecting \"BEGIN IONS\"");
        if (!t.eol()) t.fail("expecting end of line");
        // params: many (try keyval)
        std::vector<std::pair<std::string, std::string>> kv;
        while (true) {
            const size_t save = t.pos;
            while (!t.eof() && is_space((uint8_t)t.p[t.pos])) ++t.pos;
            if (t.eof() || !(is_alpha((uint8_t)t.p[t.pos]) || t.p[t.pos] == '_')) {
                t.pos = save;
                break;
            }
            const size_t k0 = t.pos;
            while (!t.eof() && (is_alpha((uint8_t)t.p[t.pos]) || is_digit((uint8_t)t.p[t.pos]) ||
                                t.p[t.pos] == '_' || t.p[t.pos] == '-'))
                ++t.pos;
            const std::string key(t.p + k0, t.pos - k0);
            while (!t.eof() && is_space((uint8_t)t.p[t.pos])) ++t.pos;
            if (t.eof() || t.p[t.pos] != '=') {
                t.pos = save;
                break;
            }
            ++t.pos;
            while (!t.eof() && is_space((uint8_t)t.p[t.pos])) ++t.pos;
            if (t.eof() || t.p[t.pos] == '#' || t.p[t.pos] == '\n' || t.p[t.pos] == '\r') {
                t.pos = save;
                break;
            }
            const size_t v0 = t.pos++;
            while (!t.eof() && t.p[t.pos] != '#' && t.p[t.pos] != '\n' && t.p[t.pos] != '\r') ++t.pos;
            size_t v1 = t.pos;
            if (!t.eof() && t.p[t.pos] == '#') {
                while (!t.eof() && t.p[t.pos] != '\n' && t.p[t.pos] != '\r') ++t.pos;  // comment, eol left
            } else {
                t.eol();
            }
            while (v1 > v0 && is_space((uint8_t)t.p[v1 - 1])) --v1;
            kv.emplace_back(key, std::string(t.p + v0, v1 - v0));
        }
        const size_t first = s.mz.size();
        float x, y;
        while (t.pair(x, y)) {
            s.mz.push_back(x);
            s.it.push_back(y);
        }
        if (!t.lit("END IONS")) t.fail("expecting \"END IONS\"");
        t.eol();  // the reference also requires it at the end of the file
        auto lookup = [&](const char *k) -> const std::string * {
            for (const auto &e : kv)
                if (e.first == k) return &e.second;
            return nullptr;
        };
        float charge = 0.0f, pepmass = 0.0f;
        const std::string *v;
        if ((v = lookup("CHARGE")) && !read_signed_float(v->data(), v->size(), charge))
            t.fail("no parse of CHARGE \"" + *v + "\"");
        if ((v = lookup("PEPMASS")) && !read_signed_float(v->data(), v->size(), pepmass))
            t.fail("no parse of PEPMASS \"" + *v + "\"");
        if (charge == 0.0f || pepmass == 0.0f) t.fail("missing charge state or peptide mass");
        v = lookup("TITLE");
        s.title.push_back(v ? *v : std::string());
        s.pcr.push_back(pepmass);
        s.z.push_back(charge);
        (void)first;
        s.off.push_back((int64_t)s.mz.size());
    }
}

// DTA.hs:35-55: endBy readF2 eol (text after the last pair is not read),
// then mkSpec.
void parse_dta(Text &t, hfx_spectra &s) {
    std::vector<float> xs, ys;
    float x, y;
    while (t.pair(x, y)) {
        xs.push_back(x);
        ys.push_back(y);
    }
    if (xs.empty()) throw Fail{"empty spectrum"};
    const float m = xs[0], c = ys[0];
    if (!(std::trunc(c) == c)) throw Fail{"invalid peptide charge state; expecting integer"};
    s.pcr.push_back((m + (c - 1.0f) * kHostH) / c);
    s.z.push_back(c);
    s.mz.insert(s.mz.end(), xs.begin() + 1, xs.end());
    s.it.insert(s.it.end(), ys.begin() + 1, ys.end());
    s.off.push_back((int64_t)s.mz.size());
    s.title.emplace_back();
}

// FASTA records (bio 0.5 mkSeqs over L.lines), laid out as makeSeqDB does.
void parse_fasta(const uint8_t *d, size_t n, hfx_proteins &out) {
    std::vector<std::pair<size_t, size_t>> lines;
    size_t a = 0;
    for (size_t i = 0; i <= n; ++i) {
        if (i == n || d[i] == '\n') {
            size_t b = i;
            if (b > a && d[b - 1] == '\r') --b;  // CR of CRLF files (the reference would keep it)
            if (b > a) lines.emplace_back(a, b);
            a = i + 1;
        }
    }
    size_t li = 0;
    while (li < lines.size()) {
        const auto h = lines[li++];
        if (d[h.first] != '>') throw Fail{"not a FASTA header: line " + std::to_string(li)};
        out.header.emplace_back((const char *)d + h.first + 1, h.second - h.first - 1);
        bool seq = true;
        while (li < lines.size() && d[lines[li].first] != '>') {
            const auto l = lines[li++];
            if (seq && is_alpha(d[l.first]))
                out.seq.insert(out.seq.end(), d + l.first, d + l.second);
            else
                seq = false;
        }
        if (out.seq.size() > 0xFFFFFFFFull) throw Fail{"database larger than 2^32 residues"};
        out.seg.push_back((uint32_t)out.seq.size());
    }
}

// ---------------------------------------------------------------- index

struct Reader {
    const uint8_t *p;
    size_t n, pos = 0;
    void need(size_t k) const {
        if (n - pos < k) throw Fail{"index: truncated at byte " + std::to_string(pos)};
    }
    uint64_t be(int bytes) {
        need((size_t)bytes);
        uint64_t v = 0;
        for (int i = 0; i < bytes; ++i) v = (v << 8) | p[pos++];
        return v;
    }
    int64_t length(size_t unit) {
        const int64_t v = (int64_t)be(8);
        if (v < 0 || (uint64_t)v > (n - pos) / (unit ? unit : 1)) throw Fail{"index: bad length"};
        return v;
    }
    std::string bytes() {
        const int64_t k = length(1);
        std::string s((const char *)p + pos, (size_t)k);
        pos += (size_t)k;
        return s;
    }
    std::vector<uint32_t> words() {
        const int64_t k = length(4);
        std::vector<uint32_t> v((size_t)k);
        for (auto &w : v) w = (uint32_t)be(4);
        return v;
    }
    // Float: (decodeFloat mantissa :: Integer, exponent :: Int)
    float real() {
        need(1);
        const uint8_t tag = p[pos++];
        double m;
        if (tag == 0) {
            m = (double)(int32_t)(uint32_t)be(4);
        } else if (tag == 1) {
            need(1);
            const uint8_t sign = p[pos++];
            const int64_t k = length(1);
            double mag = 0.0;
            for (int64_t i = k - 1; i >= 0; --i) mag = mag * 256.0 + p[pos + (size_t)i];
            pos += (size_t)k;
            m = sign == 255 ? -mag : mag;
        } else {
            throw Fail{"index: bad Integer tag"};
        }
        const int64_t e = (int64_t)be(8);
        if (e < -300 || e > 300) throw Fail{"index: bad exponent"};
        return (float)std::ldexp(m, (int)e);
    }
};

void put_be(std::vector<uint8_t> &o, uint64_t v, int bytes) {
    for (int i = bytes - 1; i >= 0; --i) o.push_back((uint8_t)(v >> (8 * i)));
}

void put_real(std::vector<uint8_t> &o, float x) {
    int32_t m = 0;
    int64_t e = 0;
    if (x != 0.0f) {
        int k;
        const float f = std::frexp(x, &k);  // x = f * 2^k, 0.5 <= |f| < 1
        m = (int32_t)std::ldexp(f, 24);
        e = (int64_t)k - 24;
    }
    o.push_back(0);
    put_be(o, (uint32_t)m, 4);
    put_be(o, (uint64_t)e, 8);
}

void parse_index(const uint8_t *d, size_t n, hfx_index &x) {
    Reader hr{d, n};
    x.options = hr.bytes();
    const std::vector<uint8_t> body = gunzip(d + hr.pos, n - hr.pos);
    Reader r{body.data(), body.size()};
    const int64_t nh = r.length(8);
    x.header.reserve((size_t)nh);
    for (int64_t i = 0; i < nh; ++i) x.header.push_back(r.bytes());
    const std::string ions = r.bytes();
    x.ions.assign(ions.begin(), ions.end());
    x.ion_seg = r.words();
    const int64_t nr = r.length(13);
    x.r.resize((size_t)nr);
    for (auto &v : x.r) v = r.real();
    x.c = r.words();
    x.n = r.words();
    x.frag_seg = r.words();
    if (x.c.size() != x.r.size() || x.n.size() != x.r.size()) throw Fail{"index: fragment arrays differ in length"};
    if (x.ion_seg.size() != x.header.size() + 1) throw Fail{"index: ion segments do not match the headers"};
}

}  // namespace

extern "C" {

int32_t hfx_parse_spectra(const char *text, int64_t n, int32_t kind, hfx_spectra **out, char *err, int32_t errcap) {
    if (!out || (!text && n > 0) || n < 0 || kind < 0 || kind > 1) return report(Fail{"bad arguments"}, err, errcap);
    *out = nullptr;
    try {
        auto *s = new hfx_spectra();
        Text t{text, (size_t)n};
        try {
            if (kind == 0) parse_dta(t, *s);
            else parse_mgf(t, *s);
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
        return 0;
    } catch (const Fail &f) {
        return report(f, err, errcap);
    }
}

int32_t hfx_read_spectra(const char *path, hfx_spectra **out, char *err, int32_t errcap) {
    try {
        const std::string name = path ? path : "";
        int32_t kind;
        if (ends_with_ci(name, ".dta")) kind = 0;
        else if (ends_with_ci(name, ".mgf")) kind = 1;
        else throw Fail{"Unsupported file type: " + name};
        const std::vector<uint8_t> d = read_file(path);
        const int32_t rc = hfx_parse_spectra((const char *)d.data(), (int64_t)d.size(), kind, out, err, errcap);
        if (rc && err && errcap > 0) {
            const std::string m = name + ": " + err;
            std::snprintf(err, (size_t)errcap, "%s", m.c_str());
        }
        return rc;
    } catch (const Fail &f) {
        return report(f, err, errcap);
    }
}

int64_t hfx_spectra_count(const hfx_spectra *s) { return s ? (int64_t)s->pcr.size() : 0; }

void hfx_spectra_arrays(const hfx_spectra *s, const float **mz, const float **it, const int64_t **off,
                        const float **pcr, const float **z) {
    if (mz) *mz = s->mz.data();
    if (it) *it = s->it.data();
    if (off) *off = s->off.data();
    if (pcr) *pcr = s->pcr.data();
    if (z) *z = s->z.data();
}

const char *hfx_spectra_title(const hfx_spectra *s, int64_t i, int64_t *len) {
    if (!s || i < 0 || (size_t)i >= s->title.size()) return nullptr;
    if (len) *len = (int64_t)s->title[(size_t)i].size();
    return s->title[(size_t)i].c_str();
}

void hfx_spectra_free(hfx_spectra *s) { delete s; }

int32_t hfx_parse_fasta(const uint8_t *data, int64_t n, int32_t gz, hfx_proteins **out, char *err, int32_t errcap) {
    if (!out || (!data && n > 0) || n < 0) return report(Fail{"bad arguments"}, err, errcap);
    *out = nullptr;
    try {
        auto *p = new hfx_proteins();
        try {
            if (gz) {
                const std::vector<uint8_t> d = gunzip(data, (size_t)n);
                parse_fasta(d.data(), d.size(), *p);
            } else {
                parse_fasta(data, (size_t)n, *p);
            }
        } catch (...) {
            delete p;
            throw;
        }
        *out = p;
        return 0;
    } catch (const Fail &f) {
        return report(f, err, errcap);
    }
}

int32_t hfx_read_fasta(const char *path, hfx_proteins **out, char *err, int32_t errcap) {
    try {
        const std::vector<uint8_t> d = read_file(path);
        const std::string name = path;
        return hfx_parse_fasta(d.data(), (int64_t)d.size(), name.size() >= 3 && name.compare(name.size() - 3, 3, ".gz") == 0,
                               out, err, errcap);
    } catch (const Fail &f) {
        return report(f, err, errcap);
    }
}

int64_t hfx_proteins_count(const hfx_proteins *p) { return p ? (int64_t)p->header.size() : 0; }

void hfx_proteins_arrays(const hfx_proteins *p, const uint8_t **seq, const uint32_t **seg) {
    if (seq) *seq = p->seq.data();
    if (seg) *seg = p->seg.data();
}

const char *hfx_proteins_header(const hfx_proteins *p, int64_t i, int64_t *len) {
    if (!p || i < 0 || (size_t)i >= p->header.size()) return nullptr;
    if (len) *len = (int64_t)p->header[(size_t)i].size();
    return p->header[(size_t)i].c_str();
}

void hfx_proteins_free(hfx_proteins *p) { delete p; }

int32_t hfx_parse_index(const uint8_t *data, int64_t n, hfx_index **out, char *err, int32_t errcap) {
    if (!out || (!data && n > 0) || n < 0) return report(Fail{"bad arguments"}, err, errcap);
    *out = nullptr;
    try {
        auto *x = new hfx_index();
        try {
            parse_index(data, (size_t)n, *x);
        } catch (...) {
            delete x;
            throw;
        }
        *out = x;
        return 0;
    } catch (const Fail &f) {
        return report(f, err, errcap);
    }
}

int32_t hfx_read_index(const char *path, hfx_index **out, char *err, int32_t errcap) {
    try {
        const std::vector<uint8_t> d = read_file(path);
        return hfx_parse_index(d.data(), (int64_t)d.size(), out, err, errcap);
    } catch (const Fail &f) {
        return report(f, err, errcap);
    }
}

const char *hfx_index_options(const hfx_index *x, int64_t *len) {
    if (len) *len = (int64_t)x->options.size();
    return x->options.c_str();
}

void hfx_index_sizes(const hfx_index *x, int64_t *num_headers, int64_t *num_ions, int64_t *num_frags) {
    if (num_headers) *num_headers = (int64_t)x->header.size();
    if (num_ions) *num_ions = (int64_t)x->ions.size();
    if (num_frags) *num_frags = (int64_t)x->r.size();
}

const char *hfx_index_header(const hfx_index *x, int64_t i, int64_t *len) {
    if (!x || i < 0 || (size_t)i >= x->header.size()) return nullptr;
    if (len) *len = (int64_t)x->header[(size_t)i].size();
    return x->header[(size_t)i].c_str();
}

void hfx_index_arrays(const hfx_index *x, const uint8_t **ions, const uint32_t **ion_seg, const float **r,
                      const uint32_t **c, const uint32_t **n, const uint32_t **frag_seg) {
    if (ions) *ions = x->ions.data();
    if (ion_seg) *ion_seg = x->ion_seg.data();
    if (r) *r = x->r.data();
    if (c) *c = x->c.data();
    if (n) *n = x->n.data();
    if (frag_seg) *frag_seg = x->frag_seg.data();
}

void hfx_index_free(hfx_index *x) { delete x; }

int32_t hfx_write_index(const char *path, const char *options, int64_t num_headers, const char *const *headers,
                        const uint8_t *ions, int64_t num_ions, const uint32_t *ion_seg, const float *r,
                        const uint32_t *c, const uint32_t *n, int64_t num_frags, const uint32_t *frag_seg,
                        char *err, int32_t errcap) {
    try {
        if (!path || !options || num_headers < 0 || num_ions < 0 || num_frags < 0 || (num_headers && !headers) ||
            (num_ions && !ions) || !ion_seg || (num_frags && (!r || !c || !n)) || !frag_seg)
            throw Fail{"bad hfx_write_index arguments"};
        std::vector<uint8_t> o;
        const size_t ol = std::strlen(options);
        put_be(o, ol, 8);
        o.insert(o.end(), options, options + ol);
        std::vector<uint8_t> b;
        put_be(b, (uint64_t)num_headers, 8);
        for (int64_t i = 0; i < num_headers; ++i) {
            const size_t k = std::strlen(headers[i]);
            put_be(b, k, 8);
            b.insert(b.end(), headers[i], headers[i] + k);
        }
        put_be(b, (uint64_t)num_ions, 8);
        b.insert(b.end(), ions, ions + num_ions);
        auto words = [&](const uint32_t *w, int64_t k) {
            put_be(b, (uint64_t)k, 8);
            for (int64_t i = 0; i < k; ++i) put_be(b, w[i], 4);
        };
        words(ion_seg, num_headers + 1);
        put_be(b, (uint64_t)num_frags, 8);
        for (int64_t i = 0; i < num_frags; ++i) put_real(b, r[i]);
        words(c, num_frags);
        words(n, num_frags);
        words(frag_seg, num_headers + 1);
        const std::vector<uint8_t> z = gzip_stored(b);
        o.insert(o.end(), z.begin(), z.end());
        FILE *fp = std::fopen(path, "wb");
        if (!fp) throw Fail{std::string("cannot create ") + path};
        const bool ok = std::fwrite(o.data(), 1, o.size(), fp) == o.size();
        if (std::fclose(fp) != 0 || !ok) throw Fail{std::string("cannot write ") + path};
        return 0;
    } catch (const Fail &f) {
        return report(f, err, errcap);
    }
}

}  // extern "C"
