// Host-side batch reads of many files (qmlg_read_files) and parse of XYZ files
// (qmlg_parse_xyz).
//
// Each file is parsed as qml/compound.py Compound.read_xyz (:296-326) parses it: the
// atom count is line 1, line 2 is a comment, and from line 3 on each line gives an
// element symbol and x, y, z; the walk stops after the counted lines, at the end of
// the file, or at a line with fewer than four whitespace-separated fields.  Lines end
// at "\n", "\r\n" or "\r" (Python's universal newlines); fields split on the ASCII
// whitespace str.split() uses.
//
// This parser reads a subset of what Python reads, and flags every other file
// instead of guessing: bytes outside ASCII (Python decodes the text first), an
// atom-count line that is not a plain decimal integer >= 0, an element missing from
// the charge table, and a number that strtod does not read in full (Python's float()
// also takes "1_0" and rejects hex and "nan(...)", so those files go back to the
// caller too).  strtod and float() both round correctly, so an accepted file gives
// the same bits.
//
// Work is split over host threads twice: phase 1 counts each file's atoms, a prefix
// sum places the files, phase 2 parses the numbers into place.
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "qmlg.h"

namespace {

// element symbols in order of nuclear charge, the table of qml/data.py:23: elements
// 1-112, then the placeholder names Uuq = 114 and Uuh = 116
const char kSymbols[] =
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge "
    "As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm "
    "Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U "
    "Np Pu Am Cm Bk Cf Es Fm Md No Lr Rf Db Sg Bh Hs Mt Ds Rg Cn Uuq Uuh";

// a symbol of up to three characters packed into one word
inline uint32_t pack(const char *s, size_t n) {
    uint32_t w = 0;
    for (size_t i = 0; i < n; ++i) w |= (uint32_t)(unsigned char)s[i] << (8 * i);
    return w;
}

struct ChargeTable {
    uint32_t key[114];
    int charge[114];
    int n = 0;
    ChargeTable() {
        const char *p = kSymbols;
        while (*p) {
            const char *b = p;
            while (*p && *p != ' ') ++p;
            key[n] = pack(b, (size_t)(p - b));
            charge[n] = n < 112 ? n + 1 : (n == 112 ? 114 : 116);
            ++n;
            while (*p == ' ') ++p;
        }
    }
};

const ChargeTable kCharges;

inline bool is_space(unsigned char c) {
    return c == ' ' || (c >= 9 && c <= 13) || (c >= 28 && c <= 31);
}

// 0 for a symbol the table does not hold
int charge_of(const char *s, size_t n) {
    if (n == 0 || n > 3) return 0;
    uint32_t w = pack(s, n);
    for (int i = 0; i < kCharges.n; ++i)
        if (kCharges.key[i] == w) return kCharges.charge[i];
    return 0;
}

// One line of [p, end): sets [b, e) and returns the start of the next line.
const char *next_line(const char *p, const char *end, const char *&b, const char *&e) {
    b = p;
    while (p < end && *p != '\n' && *p != '\r') ++p;
    e = p;
    if (p < end) {
        if (*p == '\r' && p + 1 < end && p[1] == '\n') ++p;
        ++p;
    }
    return p;
}

// Up to four fields of [b, e); returns the number of fields (stops counting at 4).
int fields(const char *b, const char *e, const char *fb[4], const char *fe[4]) {
    int n = 0;
    while (n < 4) {
        while (b < e && is_space((unsigned char)*b)) ++b;
        if (b == e) break;
        fb[n] = b;
        while (b < e && !is_space((unsigned char)*b)) ++b;
        fe[n++] = b;
    }
    return n;
}

bool parse_count(const char *b, const char *e, int64_t &n) {
    while (b < e && is_space((unsigned char)*b)) ++b;
    while (e > b && is_space((unsigned char)e[-1])) --e;
    if (b < e && *b == '+') ++b;
    if (b == e || e - b > 12) return false;
    n = 0;
    for (; b < e; ++b) {
        if (*b < '0' || *b > '9') return false;
        n = n * 10 + (*b - '0');
    }
    return true;
}

bool parse_number(const char *b, const char *e, double &v) {
    char buf[64];
    size_t n = (size_t)(e - b);
    if (n == 0 || n >= sizeof(buf)) return false;
    for (size_t i = 0; i < n; ++i) {
        char c = b[i];
        if (c == 'x' || c == 'X' || c == '(') return false;  // hex and nan(...) forms
        buf[i] = c;
    }
    buf[n] = 0;
    char *stop = nullptr;
    v = std::strtod(buf, &stop);
    return stop == buf + n;
}

// Walks the atom lines of one file.  With charges == nullptr it only counts them
// (and checks the symbols); otherwise it also writes charges and coordinates.
// Returns the atom count, or -1 when the file is not accepted.
int64_t walk(const char *p, const char *end, double *charges, double *coords) {
    for (const char *q = p; q < end; ++q)
        if ((unsigned char)*q >= 0x80) return -1;
    if (p == end) return -1;
    const char *b, *e;
    p = next_line(p, end, b, e);
    int64_t natoms;
    if (!parse_count(b, e, natoms)) return -1;
    if (p < end) p = next_line(p, end, b, e);  // the comment line
    int64_t n = 0;
    const char *fb[4], *fe[4];
    while (n < natoms && p < end) {
        p = next_line(p, end, b, e);
        if (fields(b, e, fb, fe) < 4) break;
        int z = charge_of(fb[0], (size_t)(fe[0] - fb[0]));
        if (z == 0) return -1;
        if (charges) {
            charges[n] = (double)z;
            for (int k = 0; k < 3; ++k)
                if (!parse_number(fb[k + 1], fe[k + 1], coords[3 * n + k])) return -1;
        }
        ++n;
    }
    return n;
}

template <class F>
void parallel_files(int nfiles, int nthreads, F &&fn) {
    const int chunk = 64;
    std::atomic<int> next{0};
    auto run = [&]() {
        for (;;) {
            int f0 = next.fetch_add(chunk);
            if (f0 >= nfiles) return;
            int f1 = f0 + chunk < nfiles ? f0 + chunk : nfiles;
            for (int f = f0; f < f1; ++f) fn(f);
        }
    };
    int t = nthreads;
    if (t > (nfiles + chunk - 1) / chunk) t = (nfiles + chunk - 1) / chunk;
    if (t <= 1) {
        run();
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(t - 1);
    for (int i = 1; i < t; ++i) pool.emplace_back(run);
    run();
    for (auto &th : pool) th.join();
}

}  // namespace

extern "C" int qmlg_parse_xyz(const char *text, const int64_t *starts, int nfiles, int nthreads,
                              int64_t *offsets, int *status, double *charges,
                              double *coordinates, int64_t capacity) {
    if (nfiles < 0 || !starts || !offsets || !status || capacity < 0) return QMLG_E_ARG;
    if (nfiles > 0 && (!text || ((!charges || !coordinates) && capacity > 0))) return QMLG_E_ARG;
    for (int f = 0; f < nfiles; ++f)
        if (starts[f] < 0 || starts[f + 1] < starts[f]) return QMLG_E_ARG;
    if (nthreads <= 0) {
        unsigned hc = std::thread::hardware_concurrency();
        nthreads = hc ? (int)hc : 1;
    }
    std::vector<int64_t> count(nfiles);
    parallel_files(nfiles, nthreads, [&](int f) {
        count[f] = walk(text + starts[f], text + starts[f + 1], nullptr, nullptr);
    });
    offsets[0] = 0;
    for (int f = 0; f < nfiles; ++f) {
        status[f] = count[f] < 0 ? 1 : 0;
        offsets[f + 1] = offsets[f] + (count[f] < 0 ? 0 : count[f]);
    }
    if (offsets[nfiles] > capacity) return QMLG_E_TOO_LARGE;
    parallel_files(nfiles, nthreads, [&](int f) {
        if (status[f]) return;
        int64_t o = offsets[f];
        if (walk(text + starts[f], text + starts[f + 1], charges + o, coordinates + 3 * o) < 0)
            status[f] = 1;
    });
    return QMLG_OK;
}

namespace {

// Size of a regular file, or -1.
int64_t file_size(const char *path) {
    struct stat st;
    if (stat(path, &st) != 0 || !S_ISREG(st.st_mode)) return -1;
    return (int64_t)st.st_size;
}

// Reads exactly n bytes of the file into dst, and checks that nothing follows.
bool read_exactly(const char *path, char *dst, int64_t n) {
    int fd = open(path, O_RDONLY);
    if (fd < 0) return false;
    int64_t got = 0;
    bool ok = true;
    while (got < n) {
        ssize_t r = read(fd, dst + got, (size_t)(n - got));
        if (r <= 0) {
            ok = false;
            break;
        }
        got += r;
    }
    char extra;
    if (ok && read(fd, &extra, 1) != 0) ok = false;
    close(fd);
    return ok;
}

}  // namespace

extern "C" int qmlg_read_files(const char *const *paths, int nfiles, int nthreads,
                               int64_t *sizes, char *buf, const int64_t *starts, int *status) {
    if (nfiles < 0 || (nfiles > 0 && (!paths || !sizes))) return QMLG_E_ARG;
    if (buf && (!starts || !status)) return QMLG_E_ARG;
    for (int f = 0; f < nfiles; ++f)
        if (!paths[f]) return QMLG_E_ARG;
    if (nthreads <= 0) {
        unsigned hc = std::thread::hardware_concurrency();
        nthreads = hc ? (int)hc : 1;
    }
    if (!buf) {
        parallel_files(nfiles, nthreads, [&](int f) { sizes[f] = file_size(paths[f]); });
        return QMLG_OK;
    }
    for (int f = 0; f < nfiles; ++f)
        if (starts[f] < 0 || starts[f + 1] < starts[f]) return QMLG_E_ARG;
    parallel_files(nfiles, nthreads, [&](int f) {
        int64_t n = starts[f + 1] - starts[f];
        status[f] = (sizes[f] == n && read_exactly(paths[f], buf + starts[f], n)) ? 0 : 1;
    });
    return QMLG_OK;
}
