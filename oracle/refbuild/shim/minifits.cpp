// Test-infrastructure shim (oracle build only): a minimal FITS reader/writer
// that implements the image-HDU subset of cfitsio used by lyspeq's lookup
// table files.  FITS layout (NASA/IAU FITS standard 4.0): 2880-byte blocks,
// 80-character header cards ending with END, big-endian data padded with
// zeros to a block boundary.  Table-HDU calls return status 1.
#include "fitsio.h"

#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {
struct Card { std::string key, value; bool is_string; };

struct Hdu {
    std::vector<Card> cards;     // every card except END, in file order
    std::vector<unsigned char> data;
    int bitpix = 8;
    std::vector<long> naxes;
};

std::string trim(const std::string &s) {
    size_t b = s.find_first_not_of(' '), e = s.find_last_not_of(' ');
    if (b == std::string::npos) return "";
    return s.substr(b, e - b + 1);
}

const Card *findCard(const Hdu &h, const std::string &key) {
    for (const auto &c : h.cards)
        if (c.key == key) return &c;
    return nullptr;
}

Card *findCardMut(Hdu &h, const std::string &key) {
    for (auto &c : h.cards)
        if (c.key == key) return &c;
    return nullptr;
}

std::string upper(std::string s) {
    for (auto &ch : s) ch = (char) std::toupper((unsigned char) ch);
    return s;
}
}  // namespace

struct lqg_minifits {
    std::string path;
    bool writable = false;
    std::vector<Hdu> hdus;
    int cur = 0;
};

namespace {
void parseCard(const char *c80, Card &card, bool &is_end) {
    std::string line(c80, 80);
    card.key = trim(line.substr(0, 8));
    is_end = card.key == "END";
    card.is_string = false;
    card.value.clear();
    if (line.compare(8, 2, "= ") != 0) return;
    std::string rest = line.substr(10);
    size_t p = rest.find_first_not_of(' ');
    if (p == std::string::npos) return;
    if (rest[p] == '\'') {
        card.is_string = true;
        std::string v;
        for (size_t i = p + 1; i < rest.size(); ++i) {
            if (rest[i] == '\'') {
                if (i + 1 < rest.size() && rest[i + 1] == '\'') { v += '\''; ++i; }
                else break;
            } else v += rest[i];
        }
        while (!v.empty() && v.back() == ' ') v.pop_back();
        card.value = v;
    } else {
        size_t slash = rest.find('/', p);
        card.value = trim(rest.substr(p, slash == std::string::npos ? std::string::npos : slash - p));
    }
}

long cardLong(const Hdu &h, const std::string &key, long dflt) {
    const Card *c = findCard(h, key);
    if (!c) return dflt;
    return std::strtol(c->value.c_str(), nullptr, 10);
}

bool readAll(lqg_minifits *f) {
    FILE *fp = std::fopen(f->path.c_str(), "rb");
    if (!fp) return false;
    std::vector<unsigned char> buf;
    unsigned char tmp[2880];
    size_t n;
    while ((n = std::fread(tmp, 1, sizeof(tmp), fp)) > 0)
        buf.insert(buf.end(), tmp, tmp + n);
    std::fclose(fp);

    size_t pos = 0;
    while (pos + 2880 <= buf.size()) {
        Hdu h;
        bool end = false;
        while (!end && pos + 80 <= buf.size()) {
            Card c;
            parseCard(reinterpret_cast<const char *>(&buf[pos]), c, end);
            pos += 80;
            if (!end && !c.key.empty()) h.cards.push_back(c);
        }
        if (!end) return false;
        pos = (pos + 2879) / 2880 * 2880;
        h.bitpix = (int) cardLong(h, "BITPIX", 8);
        long naxis = cardLong(h, "NAXIS", 0);
        long nelem = naxis > 0 ? 1 : 0;
        for (long i = 1; i <= naxis; ++i) {
            long ax = cardLong(h, "NAXIS" + std::to_string(i), 0);
            h.naxes.push_back(ax);
            nelem *= ax;
        }
        long pcount = cardLong(h, "PCOUNT", 0), gcount = cardLong(h, "GCOUNT", 1);
        size_t nbytes = (size_t) (std::abs(h.bitpix) / 8) * gcount * (pcount + nelem);
        if (pos + nbytes > buf.size()) return false;
        h.data.assign(buf.begin() + pos, buf.begin() + pos + nbytes);
        pos += (nbytes + 2879) / 2880 * 2880;
        f->hdus.push_back(std::move(h));
    }
    return !f->hdus.empty();
}

void putCard(std::string &out, const std::string &key, const std::string &val, bool is_string) {
    char card[81];
    std::memset(card, ' ', 80);
    card[80] = 0;
    std::memcpy(card, key.c_str(), std::min<size_t>(8, key.size()));
    if (key == "COMMENT") {
        std::memcpy(card + 8, val.c_str(), std::min<size_t>(72, val.size()));
    } else {
        card[8] = '=';
        std::string v;
        if (is_string) {
            std::string s = val;
            while (s.size() < 8) s += ' ';
            v = "'" + s + "'";
            std::memcpy(card + 10, v.c_str(), std::min<size_t>(70, v.size()));
        } else {
            v = val;
            size_t w = std::max<size_t>(20, v.size());
            std::memcpy(card + 10 + (w - v.size()), v.c_str(), std::min<size_t>(70, v.size()));
        }
    }
    out.append(card, 80);
}

bool writeAll(lqg_minifits *f) {
    FILE *fp = std::fopen(f->path.c_str(), "wb");
    if (!fp) return false;
    for (size_t ih = 0; ih < f->hdus.size(); ++ih) {
        const Hdu &h = f->hdus[ih];
        std::string hdr;
        if (ih == 0) putCard(hdr, "SIMPLE", "T", false);
        else putCard(hdr, "XTENSION", "IMAGE", true);
        putCard(hdr, "BITPIX", std::to_string(h.bitpix), false);
        putCard(hdr, "NAXIS", std::to_string(h.naxes.size()), false);
        for (size_t i = 0; i < h.naxes.size(); ++i)
            putCard(hdr, "NAXIS" + std::to_string(i + 1), std::to_string(h.naxes[i]), false);
        if (ih == 0) putCard(hdr, "EXTEND", "T", false);
        else { putCard(hdr, "PCOUNT", "0", false); putCard(hdr, "GCOUNT", "1", false); }
        for (const auto &c : h.cards) putCard(hdr, c.key, c.value, c.is_string);
        std::string endc = "END";
        endc.resize(80, ' ');
        hdr += endc;
        hdr.resize((hdr.size() + 2879) / 2880 * 2880, ' ');
        std::fwrite(hdr.data(), 1, hdr.size(), fp);
        std::vector<unsigned char> d = h.data;
        d.resize((d.size() + 2879) / 2880 * 2880, 0);
        if (!d.empty()) std::fwrite(d.data(), 1, d.size(), fp);
    }
    std::fclose(fp);
    return true;
}

double beDouble(const unsigned char *p) {
    uint64_t u = 0;
    for (int i = 0; i < 8; ++i) u = (u << 8) | p[i];
    double d;
    std::memcpy(&d, &u, 8);
    return d;
}

void putBeDouble(unsigned char *p, double d) {
    uint64_t u;
    std::memcpy(&u, &d, 8);
    for (int i = 7; i >= 0; --i) { p[i] = (unsigned char) (u & 0xff); u >>= 8; }
}

int fail(int *status, int code) { if (status) *status = code; return code; }
}  // namespace

int fits_open_file(fitsfile **fptr, const char *filename, int iomode, int *status) {
    if (*status) return *status;
    auto *f = new lqg_minifits();
    f->path = filename;
    f->writable = iomode == READWRITE;
    if (!readAll(f)) { delete f; *fptr = nullptr; return fail(status, 104); }
    *fptr = f;
    return 0;
}

int fits_create_file(fitsfile **fptr, const char *filename, int *status) {
    if (*status) return *status;
    auto *f = new lqg_minifits();
    f->path = filename[0] == '!' ? filename + 1 : filename;
    f->writable = true;
    f->cur = -1;
    *fptr = f;
    return 0;
}

int fits_close_file(fitsfile *f, int *status) {
    if (!f) return *status;
    bool ok = true;
    if (f->writable) ok = writeAll(f);
    delete f;
    if (!ok && *status == 0) *status = 106;
    return *status;
}

void fits_get_errstatus(int status, char *err_text) {
    std::snprintf(err_text, 30, "minifits status %d", status);
}

int fits_movnam_hdu(fitsfile *f, int, char *extname, int, int *status) {
    if (*status) return *status;
    std::string want = upper(trim(extname));
    for (size_t i = 0; i < f->hdus.size(); ++i) {
        const Card *c = findCard(f->hdus[i], "EXTNAME");
        if (c && upper(trim(c->value)) == want) { f->cur = (int) i; return 0; }
    }
    return fail(status, 301);
}

int fits_movabs_hdu(fitsfile *f, int hdunum, int *hdutype, int *status) {
    if (*status) return *status;
    if (hdunum < 1 || hdunum > (int) f->hdus.size()) return fail(status, 107);
    f->cur = hdunum - 1;
    if (hdutype) *hdutype = IMAGE_HDU;
    return 0;
}

int fits_get_num_hdus(fitsfile *f, int *hdunum, int *status) {
    if (*status) return *status;
    *hdunum = (int) f->hdus.size();
    return 0;
}

int fits_get_hdu_num(fitsfile *f, int *hdunum) { *hdunum = f->cur + 1; return *hdunum; }

int fits_get_hdrspace(fitsfile *f, int *keysexist, int *morekeys, int *status) {
    if (*status) return *status;
    if (keysexist) *keysexist = (int) f->hdus[f->cur].cards.size();
    if (morekeys) *morekeys = -1;
    return 0;
}

int fits_read_key(fitsfile *f, int datatype, const char *keyname, void *value, char *comm,
                  int *status) {
    if (*status) return *status;
    if (comm) comm[0] = 0;
    const Card *c = findCard(f->hdus[f->cur], upper(trim(keyname)));
    if (!c) return fail(status, 202);
    std::string v = c->value;
    for (auto &ch : v) if (ch == 'D' || ch == 'd') ch = 'E';
    switch (datatype) {
    case TINT: *static_cast<int *>(value) = (int) std::strtol(v.c_str(), nullptr, 10); break;
    case TUINT: *static_cast<unsigned *>(value) = (unsigned) std::strtoul(v.c_str(), nullptr, 10); break;
    case TLONG: *static_cast<long *>(value) = std::strtol(v.c_str(), nullptr, 10); break;
    case TLONGLONG: *static_cast<long long *>(value) = std::strtoll(v.c_str(), nullptr, 10); break;
    case TDOUBLE: *static_cast<double *>(value) = std::strtod(v.c_str(), nullptr); break;
    case TFLOAT: *static_cast<float *>(value) = (float) std::strtod(v.c_str(), nullptr); break;
    case TLOGICAL: *static_cast<int *>(value) = (trim(v) == "T"); break;
    case TSTRING: std::strcpy(static_cast<char *>(value), c->value.c_str()); break;
    default: return fail(status, 410);
    }
    return 0;
}

int fits_read_keyn(fitsfile *, int, char *, char *, char *, int *status) {
    return fail(status, 1);
}

int fits_read_keys_lng(fitsfile *f, const char *keyname, int nstart, int nmax, long *value,
                       int *nfound, int *status) {
    if (*status) return *status;
    *nfound = 0;
    for (int i = nstart; i < nstart + nmax; ++i) {
        const Card *c = findCard(f->hdus[f->cur], upper(keyname) + std::to_string(i));
        if (!c) continue;
        value[i - nstart] = std::strtol(c->value.c_str(), nullptr, 10);
        *nfound = i - nstart + 1;
    }
    return 0;
}

int fits_make_keyn(const char *keyroot, int value, char *keyname, int *status) {
    if (*status) return *status;
    std::snprintf(keyname, FLEN_KEYWORD, "%s%d", keyroot, value);
    return 0;
}

int fits_get_num_cols(fitsfile *, int *, int *status) { return fail(status, 1); }
int fits_get_num_rows(fitsfile *, long *, int *status) { return fail(status, 1); }
int fits_get_colnum(fitsfile *, int, char *, int *, int *status) { return fail(status, 1); }
int fits_read_col(fitsfile *, int, int, LONGLONG, LONGLONG, LONGLONG, void *, void *, int *,
                  int *status) { return fail(status, 1); }
int fits_read_tdim(fitsfile *, int, int, int *, long *, int *status) { return fail(status, 1); }

int fits_create_img(fitsfile *f, int bitpix, int naxis, long *naxes, int *status) {
    if (*status) return *status;
    if (bitpix != DOUBLE_IMG) return fail(status, 410);
    Hdu h;
    h.bitpix = bitpix;
    long nelem = naxis > 0 ? 1 : 0;
    for (int i = 0; i < naxis; ++i) { h.naxes.push_back(naxes[i]); nelem *= naxes[i]; }
    h.data.assign((size_t) nelem * 8, 0);
    f->hdus.push_back(std::move(h));
    f->cur = (int) f->hdus.size() - 1;
    return 0;
}

int fits_write_img(fitsfile *f, int datatype, LONGLONG firstelem, LONGLONG nelem, void *array,
                   int *status) {
    if (*status) return *status;
    if (datatype != TDOUBLE) return fail(status, 410);
    Hdu &h = f->hdus[f->cur];
    if ((size_t) (firstelem - 1 + nelem) * 8 > h.data.size()) return fail(status, 308);
    const double *a = static_cast<const double *>(array);
    for (LONGLONG i = 0; i < nelem; ++i) putBeDouble(&h.data[(firstelem - 1 + i) * 8], a[i]);
    return 0;
}

int fits_read_img(fitsfile *f, int datatype, LONGLONG firstelem, LONGLONG nelem, void *,
                  void *array, int *anynul, int *status) {
    if (*status) return *status;
    if (anynul) *anynul = 0;
    const Hdu &h = f->hdus[f->cur];
    if (datatype != TDOUBLE || h.bitpix != DOUBLE_IMG) return fail(status, 410);
    if ((size_t) (firstelem - 1 + nelem) * 8 > h.data.size()) return fail(status, 308);
    double *a = static_cast<double *>(array);
    for (LONGLONG i = 0; i < nelem; ++i) a[i] = beDouble(&h.data[(firstelem - 1 + i) * 8]);
    return 0;
}

int fits_write_key(fitsfile *f, int datatype, const char *keyname, void *value, const char *,
                   int *status) {
    if (*status) return *status;
    char buf[64];
    bool is_string = false;
    switch (datatype) {
    case TINT: std::snprintf(buf, sizeof buf, "%d", *static_cast<int *>(value)); break;
    case TUINT: std::snprintf(buf, sizeof buf, "%u", *static_cast<unsigned *>(value)); break;
    case TLONG: std::snprintf(buf, sizeof buf, "%ld", *static_cast<long *>(value)); break;
    case TDOUBLE: std::snprintf(buf, sizeof buf, "%.17G", *static_cast<double *>(value)); break;
    case TLOGICAL: std::snprintf(buf, sizeof buf, "%s", *static_cast<int *>(value) ? "T" : "F"); break;
    case TSTRING: std::snprintf(buf, sizeof buf, "%s", static_cast<char *>(value)); is_string = true; break;
    default: return fail(status, 410);
    }
    Hdu &h = f->hdus[f->cur];
    std::string key = upper(keyname);
    Card *c = findCardMut(h, key);
    if (c) { c->value = buf; c->is_string = is_string; }
    else h.cards.push_back({key, buf, is_string});
    return 0;
}

int fits_update_key_str(fitsfile *f, const char *keyname, const char *value, const char *,
                        int *status) {
    if (*status) return *status;
    Hdu &h = f->hdus[f->cur];
    std::string key = upper(keyname);
    Card *c = findCardMut(h, key);
    if (c) { c->value = value; c->is_string = true; }
    else h.cards.push_back({key, value, true});
    return 0;
}

int fits_write_comment(fitsfile *f, const char *comment, int *status) {
    if (*status) return *status;
    f->hdus[f->cur].cards.push_back({"COMMENT", comment, false});
    return 0;
}
