// host_params.cpp -- run parameters and initial state on the host.
//
// gm_params_default / gm_params_derive / gm_params_read restate the Fortran
// namelist reader src/readNamelist.f90 (defaults :92-150, namelists :152-171,
// derived grid spacing :185-186, string copy :267-283).  gm_init_state
// restates initState/initDistortion (src/init.cu:30-419) for the initial
// fields the relaxation benchmarks use, and the periodic B0 copy
// setPeriHost (src/boundaries.cu:492-528).
#include <cctype>
#include <cerrno>
#include <climits>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "glemur.h"
#include "gm_internal.h"

namespace {

// Fortran default initialisers such as `dt0 = 3e-4` are default-kind (single
// precision) literals converted to the variable's kind, so in a PRECISION=64
// build the default is the float value widened to double.
double flit(double v) { return (double)(float)v; }

void set_str(char* dst, const char* src) {
    // blank padded to 29 characters plus NUL, as copyString leaves it
    size_t n = strlen(src);
    for (int i = 0; i < GM_STR_LEN - 1; i++) dst[i] = (size_t)i < n ? src[i] : ' ';
    dst[GM_STR_LEN - 1] = '\0';
}

}  // namespace

extern "C" int gm_params_default(gm_params* p, int precision) {
    if (!p || (precision != 32 && precision != 64)) return gm::fail(GM_EPARAM, "gm_params_default: precision must be 32 or 64");
    memset(p, 0, sizeof(*p));
    p->precision = precision;
    p->nx = 16; p->ny = 16; p->nz = 16;
    p->Lx = 8.; p->Ly = 8.; p->Lz = 20.;
    p->Ox = 0.; p->Oy = 0.; p->Oz = 0.;
    set_str(p->bInit, "Pontin09");
    set_str(p->uInit, "nil");
    p->ampl = 1.;
    p->phi1 = 2.; p->phi2 = -2.;
    p->L1 = -4.; p->L2 = 4.;
    p->ar = flit(1.414213562373095); p->az = 2.;
    p->nBlobs = 0;
    p->width = flit(0.6);
    p->minor = 1.0; p->major = 2.5;
    p->stretch = 1.0;
    p->bGround = 0.;
    set_str(p->initDist, "none");
    p->initDistCode = 0;   // never assigned for "none"; the C struct is zero-initialised
    p->initShearA = 0.; p->initShearB = 0.; p->initShearK = 1.;
    p->pert = 1.; p->twist = 1.;
    p->fRestart = 0;
    p->nCycle = 10;
    p->dt0 = flit(3e-4);
    p->dtMin = flit(1e-9);
    p->maxError = flit(5e-5);
    p->zUpdate = 1; p->inertia = 0; p->pressure = 0;
    p->nu = 1; p->beta = 1;
    p->jxbAver = 0; p->jxbAverWeight = 0.;
    p->xPeri = 0; p->yPeri = 0; p->zPeri = 0;
    p->epsilonProf = 1;
    set_str(p->jMethod, "Stokes");
    set_str(p->pMethod, "Classic");
    p->nTs = 10;
    p->dtDump = 10.; p->dtSave = 1.;
    // extensions
    p->errMode = precision == 32 ? 1 : 0;
    p->p0Amp = 0.;
    p->p0Width = 2.;
    if (precision == 32) {
        // a float literal is already exact in float
        p->ar = (double)(float)p->ar;
    }
    return gm_params_derive(p);
}

extern "C" int gm_params_derive(gm_params* p) {
    if (!p) return gm::fail(GM_EPARAM, "gm_params_derive: null params");
    if (p->nx < 2 || p->ny < 2 || p->nz < 2) return gm::fail(GM_EPARAM, "gm_params_derive: nx, ny, nz must be >= 2");
    if (p->precision == 32) {
        float Lx = (float)p->Lx, Ly = (float)p->Ly, Lz = (float)p->Lz;
        float dx = Lx / (float)(p->nx - 1), dy = Ly / (float)(p->ny - 1), dz = Lz / (float)(p->nz - 1);
        p->dx = dx; p->dy = dy; p->dz = dz;
        p->dx1 = 1.0f / dx; p->dy1 = 1.0f / dy; p->dz1 = 1.0f / dz;
    } else if (p->precision == 64) {
        p->dx = p->Lx / (double)(p->nx - 1); p->dy = p->Ly / (double)(p->ny - 1); p->dz = p->Lz / (double)(p->nz - 1);
        p->dx1 = 1.0 / p->dx; p->dy1 = 1.0 / p->dy; p->dz1 = 1.0 / p->dz;
    } else {
        return gm::fail(GM_EPARAM, "gm_params_derive: precision must be 32 or 64");
    }
    return GM_OK;
}

// ---------------------------------------------------------------------------
// Namelist reader.  Accepts Fortran namelist input as gfortran reads it for
// this file: `&group ... /`, `name = v1, v2`, `name(i) = v`, repeat counts
// `r*v`, `!` comments, ',' ';' and blanks as separators, logicals starting
// with an optional '.' then T or F, quoted strings, and d/D exponents.
// ---------------------------------------------------------------------------
namespace {

struct Field {
    const char* name;
    char kind;      // 'i' int32, 'r' real, 'l' logical, 's' string
    size_t off;
    int count;
};

#define F_(nm, kd, cnt) {#nm, kd, offsetof(gm_params, nm), cnt}
const Field kComp[] = {F_(nx, 'i', 1), F_(ny, 'i', 1), F_(nz, 'i', 1)};
const Field kStart[] = {
    F_(Lx, 'r', 1), F_(Ly, 'r', 1), F_(Lz, 'r', 1), F_(Ox, 'r', 1), F_(Oy, 'r', 1), F_(Oz, 'r', 1),
    F_(bInit, 's', 1), F_(uInit, 's', 1), F_(ampl, 'r', 1), F_(phi1, 'r', 1), F_(phi2, 'r', 1),
    F_(L1, 'r', 1), F_(L2, 'r', 1), F_(ar, 'r', 1), F_(az, 'r', 1), F_(nBlobs, 'i', 1),
    F_(blobXc, 'r', 10), F_(blobYc, 'r', 10), F_(blobZc, 'r', 10), F_(blobZl, 'r', 10),
    F_(blobTwist, 'r', 10), F_(blobScale, 'r', 10), F_(width, 'r', 1), F_(minor, 'r', 1),
    F_(major, 'r', 1), F_(stretch, 'r', 1), F_(bGround, 'r', 1), F_(initDist, 's', 1),
    F_(initShearA, 'r', 1), F_(initShearB, 'r', 1), F_(initShearK, 'r', 1), F_(pert, 'r', 1),
    F_(twist, 'r', 1), F_(fRestart, 'l', 1)};
const Field kRun[] = {
    F_(nCycle, 'i', 1), F_(dt0, 'r', 1), F_(dtMin, 'r', 1), F_(maxError, 'r', 1), F_(zUpdate, 'l', 1),
    F_(inertia, 'l', 1), F_(pressure, 'l', 1), F_(nu, 'r', 1), F_(beta, 'r', 1), F_(jxbAver, 'l', 1),
    F_(jxbAverWeight, 'r', 1), F_(xPeri, 'l', 1), F_(yPeri, 'l', 1), F_(zPeri, 'l', 1),
    F_(epsilonProf, 'l', 1), F_(jMethod, 's', 1), F_(pMethod, 's', 1),
    // extensions of this library (absent from reference files, so harmless)
    F_(errMode, 'i', 1), F_(p0Amp, 'r', 1), F_(p0Width, 'r', 1), F_(stageKernel, 'i', 1)};
const Field kIo[] = {
    F_(nTs, 'i', 1), F_(dtDump, 'r', 1), F_(dtSave, 'r', 1), F_(dumpJ, 'l', 1), F_(dumpDetJac, 'l', 1),
    F_(dumpCellVol, 'l', 1), F_(dumpConvexity, 'l', 1), F_(dumpWedgeMin, 'l', 1), F_(redB2, 'l', 1),
    F_(redB2f, 'l', 1), F_(redBMax, 'l', 1), F_(redJMax, 'l', 1), F_(redJxB_B2Max, 'l', 1),
    F_(redEpsilonStar, 'l', 1), F_(redErrB_1ez, 'l', 1), F_(redErrXb_XbAn, 'l', 1), F_(redConvex, 'l', 1),
    F_(redWedgeMin, 'l', 1), F_(redU2, 'l', 1), F_(redUMax, 'l', 1)};
#undef F_

struct Group {
    const char* name;
    const Field* fields;
    size_t n;
};
const Group kGroups[] = {{"comp", kComp, sizeof(kComp) / sizeof(Field)},
                         {"start", kStart, sizeof(kStart) / sizeof(Field)},
                         {"run", kRun, sizeof(kRun) / sizeof(Field)},
                         {"io", kIo, sizeof(kIo) / sizeof(Field)}};

bool ieq(const std::string& a, const char* b) {
    size_t n = strlen(b);
    if (a.size() != n) return false;
    for (size_t i = 0; i < n; i++)
        if (tolower((unsigned char)a[i]) != tolower((unsigned char)b[i])) return false;
    return true;
}

// Strip comments (outside quotes) so the tokenizer sees only data.
std::string strip_comments(const std::string& s) {
    std::string out;
    char q = 0;
    bool comment = false;
    for (char c : s) {
        if (comment) {
            if (c == '\n') { comment = false; out += c; }
            continue;
        }
        if (q) {
            out += c;
            if (c == q) q = 0;
            continue;
        }
        if (c == '"' || c == '\'') { q = c; out += c; continue; }
        if (c == '!') { comment = true; continue; }
        out += c;
    }
    return out;
}

struct Tok {
    std::string text;
    bool quoted;
};

class Parser {
  public:
    Parser(const std::string& body, gm_params* p, const Group& g) : s_(body), p_(p), g_(g) {}

    int run(std::string* err) {
        // body between '&group' and the terminating '/'
        size_t i = 0;
        while (true) {
            skip_sep(i);
            if (i >= s_.size()) return 0;
            // name or name(index)
            size_t st = i;
            while (i < s_.size() && (isalnum((unsigned char)s_[i]) || s_[i] == '_')) i++;
            std::string name = s_.substr(st, i - st);
            if (name.empty()) { *err = "unexpected character in namelist &" + std::string(g_.name); return -1; }
            int index = 1;
            skip_blank(i);
            if (i < s_.size() && s_[i] == '(') {
                size_t e = s_.find(')', i);
                if (e == std::string::npos) { *err = "unterminated index for " + name; return -1; }
                if (!parse_int(s_.substr(i + 1, e - i - 1), &index)) { *err = "bad index for " + name; return -1; }
                i = e + 1;
                skip_blank(i);
            }
            if (i >= s_.size() || s_[i] != '=') { *err = "expected '=' after " + name; return -1; }
            i++;
            const Field* f = nullptr;
            for (size_t k = 0; k < g_.n; k++)
                if (ieq(name, g_.fields[k].name)) f = &g_.fields[k];
            if (!f) { *err = "unknown name '" + name + "' in namelist &" + std::string(g_.name); return -1; }
            // values until the next "name =" or end
            std::vector<Tok> vals;
            while (true) {
                skip_sep(i);
                if (i >= s_.size()) break;
                if (next_is_name(i)) break;
                Tok t;
                if (!read_value(i, &t, err)) return -1;
                // repeat count r*v
                size_t star = t.quoted ? std::string::npos : t.text.find('*');
                if (star != std::string::npos && star > 0 &&
                    strspn(t.text.c_str(), "0123456789") == star) {
                    // a repeat count r >= 1 that fits the array (checked before
                    // expanding it, so a huge count cannot run away)
                    int r = 0;
                    if (!parse_int(t.text.substr(0, star), &r) || r < 1 || vals.size() + (size_t)r > (size_t)f->count) {
                        *err = "bad repeat count or too many values for " + name;
                        return -1;
                    }
                    Tok v{t.text.substr(star + 1), false};
                    for (int k = 0; k < r; k++) vals.push_back(v);
                } else {
                    vals.push_back(t);
                }
            }
            if (vals.empty()) { *err = "no value for " + name; return -1; }
            if (index < 1 || index - 1 + (int)vals.size() > f->count) {
                *err = "too many values or bad index for " + name;
                return -1;
            }
            for (size_t k = 0; k < vals.size(); k++)
                if (!assign(f, index - 1 + (int)k, vals[k], err)) return -1;
        }
    }

  private:
    // a whole decimal integer within the int32 range (an out-of-range value
    // is an error, as in the Fortran reader)
    static bool parse_int(const std::string& text, int* out) {
        const char* c = text.c_str();
        while (isspace((unsigned char)*c)) c++;
        char* e = nullptr;
        errno = 0;
        const long long v = strtoll(c, &e, 10);
        while (e && isspace((unsigned char)*e)) e++;
        if (e == c || *e || errno == ERANGE || v < INT32_MIN || v > INT32_MAX) return false;
        *out = (int)v;
        return true;
    }
    void skip_blank(size_t& i) {
        while (i < s_.size() && isspace((unsigned char)s_[i])) i++;
    }
    void skip_sep(size_t& i) {
        while (i < s_.size() && (isspace((unsigned char)s_[i]) || s_[i] == ',' || s_[i] == ';')) i++;
    }
    bool next_is_name(size_t i) {
        if (!(isalpha((unsigned char)s_[i]) || s_[i] == '_')) return false;
        size_t j = i;
        while (j < s_.size() && (isalnum((unsigned char)s_[j]) || s_[j] == '_')) j++;
        skip_blank(j);
        if (j < s_.size() && s_[j] == '(') {
            size_t e = s_.find(')', j);
            if (e == std::string::npos) return false;
            j = e + 1;
            skip_blank(j);
        }
        return j < s_.size() && s_[j] == '=';
    }
    bool read_value(size_t& i, Tok* t, std::string* err) {
        if (s_[i] == '"' || s_[i] == '\'') {
            char q = s_[i++];
            std::string v;
            while (i < s_.size()) {
                if (s_[i] == q) {
                    if (i + 1 < s_.size() && s_[i + 1] == q) { v += q; i += 2; continue; }
                    i++;
                    break;
                }
                v += s_[i++];
            }
            t->text = v;
            t->quoted = true;
            return true;
        }
        size_t st = i;
        while (i < s_.size() && !isspace((unsigned char)s_[i]) && s_[i] != ',' && s_[i] != ';') {
            if (s_[i] == '"' || s_[i] == '\'') break;
            i++;
        }
        t->text = s_.substr(st, i - st);
        t->quoted = false;
        if (t->text.empty()) { *err = "empty value"; return false; }
        return true;
    }
    bool assign(const Field* f, int k, const Tok& t, std::string* err) {
        char* base = reinterpret_cast<char*>(p_) + f->off;
        switch (f->kind) {
            case 'i': {
                int v = 0;
                if (t.quoted || !parse_int(t.text, &v)) { *err = std::string("bad integer for ") + f->name + ": " + t.text; return false; }
                reinterpret_cast<int32_t*>(base)[k] = v;
                return true;
            }
            case 'r': {
                std::string v = t.text;
                for (char& c : v)
                    if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
                char* e = nullptr;
                double d;
                errno = 0;
                if (p_->precision == 32) d = (double)strtof(v.c_str(), &e);  // read straight into REAL
                else d = strtod(v.c_str(), &e);
                // an overflowing value is an error, as in the Fortran reader
                const bool overflow = errno == ERANGE && std::isinf(d);
                if (t.quoted || *e || e == v.c_str() || overflow) {
                    *err = std::string("bad real for ") + f->name + ": " + t.text;
                    return false;
                }
                reinterpret_cast<double*>(base)[k] = d;
                return true;
            }
            case 'l': {
                const char* c = t.text.c_str();
                if (*c == '.') c++;
                char ch = (char)toupper((unsigned char)*c);
                if (t.quoted || (ch != 'T' && ch != 'F')) { *err = std::string("bad logical for ") + f->name + ": " + t.text; return false; }
                reinterpret_cast<int32_t*>(base)[k] = ch == 'T';
                return true;
            }
            case 's': {
                set_str(base, t.text.c_str());
                return true;
            }
        }
        return false;
    }

    const std::string& s_;
    gm_params* p_;
    const Group& g_;
};

}  // namespace

extern "C" int gm_params_read(gm_params* p, const char* path, int precision) {
    int rc = gm_params_default(p, precision);
    if (rc) return rc;
    FILE* f = fopen(path, "rb");
    if (!f) return gm::fail(GM_EIO, std::string("gm_params_read: cannot open ") + path);
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
    fclose(f);
    text = strip_comments(text);
    size_t pos = 0;
    for (const Group& g : kGroups) {
        // find "&group" (case-insensitive) at or after pos
        size_t found = std::string::npos;
        for (size_t i = text.find('&', pos); i != std::string::npos; i = text.find('&', i + 1)) {
            size_t j = i + 1;
            size_t st = j;
            while (j < text.size() && (isalnum((unsigned char)text[j]) || text[j] == '_')) j++;
            if (ieq(text.substr(st, j - st), g.name)) { found = j; break; }
        }
        if (found == std::string::npos)
            return gm::fail(GM_EIO, std::string("gm_params_read: namelist &") + g.name + " not found in " + path);
        // terminator: '/' outside quotes
        size_t i = found;
        char q = 0;
        for (; i < text.size(); i++) {
            char c = text[i];
            if (q) { if (c == q) q = 0; continue; }
            if (c == '"' || c == '\'') { q = c; continue; }
            if (c == '/') break;
        }
        if (i >= text.size()) return gm::fail(GM_EIO, std::string("gm_params_read: unterminated namelist &") + g.name);
        std::string body = text.substr(found, i - found);
        std::string err;
        Parser ps(body, p, g);
        if (ps.run(&err) != 0) return gm::fail(GM_EIO, "gm_params_read: " + err);
        pos = i + 1;
    }
    // src/readNamelist.f90:257-262
    if (strncmp(p->initDist, "initShearX ", 11) == 0) p->initDistCode = 0;
    if (strncmp(p->initDist, "centerShift ", 12) == 0) p->initDistCode = 1;
    return gm_params_derive(p);
}

// ---------------------------------------------------------------------------
// Initial state.
// ---------------------------------------------------------------------------
namespace {

template <typename T>
T rexp(T v);
template <>
float rexp<float>(float v) { return expf(v); }
template <>
double rexp<double>(double v) { return exp(v); }

// initDistortion, src/init.cu:386-420: the grid, ghosts included; B0 refers
// to the undistorted grid.  "initShearX" shears y by a sine of x, then x by a
// sine of the sheared y, both growing linearly in z.  PI is a double constant
// (global.h:17), so the sine's argument and the product are double and only
// the stored position rounds to the run precision.  "centerShift" moves y by
// a Gaussian in x, with the constant 5.0804508111226507 (the ghost-plane
// correction addDist, boundaries.cu:26-29, uses 0.15366 instead).
template <typename T>
void init_distortion(const gm_params* g, T* xb) {
    const bool shear = strncmp(g->initDist, "initShearX ", 11) == 0;
    const bool shift = strncmp(g->initDist, "centerShift ", 12) == 0;
    if (!shear && !shift) return;
    const double kPi = 3.141592653589793;
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const T dx = (T)g->dx, dy = (T)g->dy, dz = (T)g->dz, Ox = (T)g->Ox, Oy = (T)g->Oy, Oz = (T)g->Oz;
    const T Lx = (T)g->Lx, Ly = (T)g->Ly;
    const T A = (T)g->initShearA, B = (T)g->initShearB, K = (T)g->initShearK;
    for (int k = 0; k < nz + 2; k++) {
        const T z = dz * (T)(k - 1) + Oz;
        for (int j = 0; j < ny + 2; j++) {
            const T y = dy * (T)(j - 1) + Oy;
            for (int i = 0; i < nx + 2; i++) {
                const T x = dx * (T)(i - 1) + Ox;
                T* xp = &xb[3 * ((size_t)i + (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * (size_t)k))];
                if (shear) {
                    xp[1] = (T)(xp[1] - A * std::sin(K * 2 * kPi * (x + Ox - dx / 2) / (Lx + dx)) * z);
                    const T yy = xp[1];
                    xp[0] = (T)(xp[0] - B * std::sin(K * 2 * kPi * (yy + Oy - dy / 2) / (Ly + dy)) * z);
                }
                if (shift)
                    xp[1] = (T)(xp[1] + A * rexp<T>(-K * x * x) * (1 - y * y) * (rexp<T>(-1 * z + 1) - 5.0804508111226507));
            }
        }
    }
}

template <typename T>
int init_state_t(const gm_params* g, T* B0, T* xb) {
    int mode;
    if (strncmp(g->bInit, "blobs ", 6) == 0) mode = 0;
    else if (strncmp(g->bInit, "homZ ", 5) == 0) mode = 1;
    else if (strncmp(g->bInit, "analytic ", 9) == 0) mode = 2;
    else return gm::fail(GM_EPARAM, "gm_init_state: bInit must be blobs, homZ or analytic");
    if (strncmp(g->initDist, "none ", 5) != 0 && strncmp(g->initDist, "initShearX ", 11) != 0 &&
        strncmp(g->initDist, "centerShift ", 12) != 0)
        return gm::fail(GM_EPARAM, "gm_init_state: initDist must be none, initShearX or centerShift");
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const T dx = (T)g->dx, dy = (T)g->dy, dz = (T)g->dz, Ox = (T)g->Ox, Oy = (T)g->Oy, Oz = (T)g->Oz;
    const T ampl = (T)g->ampl, ar = (T)g->ar, az = (T)g->az, phi1 = (T)g->phi1;
    auto G = [&](int i, int j, int k) { return (size_t)i + (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * (size_t)k); };
    for (int k = 0; k < nz + 2; k++) {
        T z = dz * (T)(k - 1) + Oz;
        for (int j = 0; j < ny + 2; j++) {
            T y = dy * (T)(j - 1) + Oy;
            for (int i = 0; i < nx + 2; i++) {
                T x = dx * (T)(i - 1) + Ox;
                T* Bp = &B0[3 * G(i, j, k)];
                T* xp = &xb[3 * G(i, j, k)];
                if (mode == 2) {
                    T e = rexp<T>(-(x * x + y * y) / (ar * ar) - z * z / (az * az));
                    Bp[0] = 2 * ampl * z * e * phi1 / (az * az) * y;
                    Bp[1] = -2 * ampl * z * e * phi1 / (az * az) * x;
                    Bp[2] = ampl;
                } else if (mode == 1) {
                    Bp[0] = 0; Bp[1] = 0; Bp[2] = ampl;
                } else {
                    Bp[0] = 0; Bp[1] = 0; Bp[2] = 0;
                    for (int b = 0; b < g->nBlobs && b < GM_MAX_BLOBS; b++) {
                        const T xc = (T)g->blobXc[b], yc = (T)g->blobYc[b], zc = (T)g->blobZc[b];
                        const T zl = (T)g->blobZl[b], tw = (T)g->blobTwist[b], sc = (T)g->blobScale[b];
                        T e = rexp<T>((-(x - xc) * (x - xc) - (y - yc) * (y - yc)) / (sc * sc) - (z - zc) * (z - zc) / (zl * zl));
                        Bp[0] += 2 * ampl * tw / sc * e * (-(y - yc));
                        Bp[1] += 2 * ampl * tw / sc * e * (x - xc);
                    }
                    Bp[2] = ampl;
                }
                xp[0] = x; xp[1] = y; xp[2] = z;
            }
        }
    }
    init_distortion<T>(g, xb);
    // setPeriHost (boundaries.cu:492-528), order z, y, x.  The grid keeps its
    // identity ghosts: the reference's setGridPeriHost changes no in-bounds
    // value (its shifted-component statements fall outside the inner loop).
    if (g->zPeri)
        for (int i = 0; i < nx + 2; i++)
            for (int j = 0; j < ny + 2; j++)
                for (int l = 0; l < 3; l++) {
                    B0[3 * G(i, j, 0) + l] = B0[3 * G(i, j, nz) + l];
                    B0[3 * G(i, j, nz + 1) + l] = B0[3 * G(i, j, 1) + l];
                }
    if (g->yPeri)
        for (int i = 0; i < nx + 2; i++)
            for (int k = 0; k < nz + 2; k++)
                for (int l = 0; l < 3; l++) {
                    B0[3 * G(i, 0, k) + l] = B0[3 * G(i, ny, k) + l];
                    B0[3 * G(i, ny + 1, k) + l] = B0[3 * G(i, 1, k) + l];
                }
    if (g->xPeri)
        for (int j = 0; j < ny + 2; j++)
            for (int k = 0; k < nz + 2; k++)
                for (int l = 0; l < 3; l++) {
                    B0[3 * G(0, j, k) + l] = B0[3 * G(nx, j, k) + l];
                    B0[3 * G(nx + 1, j, k) + l] = B0[3 * G(1, j, k) + l];
                }
    return GM_OK;
}

}  // namespace

extern "C" int gm_init_state(const gm_params* p, void* B0, void* xb) {
    if (!p || !B0 || !xb) return gm::fail(GM_EPARAM, "gm_init_state: null argument");
    if (p->precision == 32) return init_state_t<float>(p, (float*)B0, (float*)xb);
    if (p->precision == 64) return init_state_t<double>(p, (double*)B0, (double*)xb);
    return gm::fail(GM_EPARAM, "gm_init_state: precision must be 32 or 64");
}
