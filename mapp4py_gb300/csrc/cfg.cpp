// AtomEye CFG snapshots: reading (md.atoms.import_cfg) and writing
// (md.export_cfg), host code behind the C ABI.
//
// Reading follows ImportCFG (import_cfg.cpp): the header rules of
// read_header (32-191), the two body layouts of read_body_ext (196-372) and
// read_body_std (377-478), and the conversion of ImportCFGMD::operator()
// (496-595).  Writing follows ExportCFGMD::write_header/write_body
// (export_cfg_md.cpp:26-113).  The box arithmetic uses the reference's
// operation order (xmath.h: MSQ_2_MLT 1849-1884, MLT_inv 1403-1450, S2X and
// X2S 2636-2722), so a file read here gives the same bits as the reference.
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "internal.h"

struct mappg_cfg {
    int natoms = 0;
    bool has_vel = false;
    double H[3][3] = {};
    std::vector<double> x, v;  // [natoms][3]
    std::vector<uint8_t> elem;
    std::vector<double> masses;
    std::vector<std::string> names;
};

namespace mappg {
namespace {

[[noreturn]] void file_error(const std::string& msg) { throw Error{MAPPG_ERR_FILE, msg}; }

// The file's lines.  Only lines ended by a newline are seen: the reference
// reads with std::getline and stops at end-of-file, so an unterminated last
// line is never processed (FileReader::operator(), import.cpp:92-120).
std::vector<std::string> read_lines(const char* path) {
    FILE* fp = fopen(path, "rb");
    if (!fp) file_error(std::string("failed to open ") + path);
    std::string all;
    char buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), fp)) > 0) all.append(buf, got);
    fclose(fp);
    std::vector<std::string> lines;
    size_t p = 0;
    while (true) {
        size_t q = all.find('\n', p);
        if (q == std::string::npos) break;
        lines.emplace_back(all, p, q - p);
        p = q + 1;
    }
    return lines;
}

// Drop everything from '#' on, collapse whitespace runs to one space and
// trim; returns the number of words (FileReader::hash_remover,
// import.cpp:156-196).
int normalise(std::string& line) {
    size_t cut = line.find('#');
    if (cut != std::string::npos) line.resize(cut);
    std::string out;
    int words = 0;
    size_t i = 0, n = line.size();
    while (i < n) {
        while (i < n && isspace((unsigned char)line[i])) i++;
        if (i == n) break;
        if (words) out.push_back(' ');
        words++;
        while (i < n && !isspace((unsigned char)line[i])) out.push_back(line[i++]);
    }
    line.swap(out);
    return words;
}

// whitespace-separated words of a normalised line
std::vector<const char*> words_of(std::string& line) {
    std::vector<const char*> w;
    char* p = &line[0];
    char* end = p + line.size();
    while (p < end) {
        w.push_back(p);
        while (p < end && *p != ' ') p++;
        if (p < end) *p++ = '\0';
    }
    return w;
}

// symmetric positive-definite 3x3 square root from the invariants of A
// (L. P. Franca, Computers Math. Applic. 18(5), 459-466, 1989); false when
// A is not positive definite
bool spd_sqrt3(const double A[3][3], double R[3][3]) {
    double I1 = A[0][0] + A[1][1] + A[2][2];
    double tr2 = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) tr2 += A[i][j] * A[j][i];
    double I2 = 0.5 * (I1 * I1 - tr2);
    double I3 = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    double k = I1 * I1 - 3.0 * I2;
    // a negative determinant is refused too (the invariant test alone lets
    // it through to a NaN square root)
    if (k < 0.0 || I3 <= 0.0) return false;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) R[i][j] = 0.0;
    if (k < 1e-10) {  // A is a multiple of the identity
        if (I1 <= 0.0) return false;
        for (int i = 0; i < 3; i++) R[i][i] = sqrt(I1 / 3.0);
        return true;
    }
    double l = I1 * (I1 * I1 - 4.5 * I2) + 13.5 * I3;
    double c = l / (k * sqrt(k));
    if (c > 1.0 || c < -1.0) return false;
    // largest eigenvalue of A, then the invariants of sqrt(A)
    double lam = sqrt((I1 + 2.0 * sqrt(k) * cos(acos(c) / 3.0)) / 3.0);
    double J3 = sqrt(I3);
    double y = I1 - lam * lam + 2.0 * J3 / lam;
    if (y < 0.0) return false;
    double J1 = lam + sqrt(y);
    double J2 = 0.5 * (J1 * J1 - I1);
    double den = J1 * J2 - J3;
    if (den == 0.0) return false;
    // sqrt(A) = (-A^2 + (J1^2 - J2) A + J1 J3 I) / (J1 J2 - J3)
    double inv = 1.0 / den;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double a2 = 0.0;
            for (int q = 0; q < 3; q++) a2 += A[i][q] * A[q][j];
            R[i][j] = inv * (-a2 + (J1 * J1 - J2) * A[i][j] + (i == j ? J1 * J3 : 0.0));
        }
    return true;
}

// right-nested dot product a0 b0 + (a1 b1 + (... )) of n terms, the order of
// the reference's __V_mul_V (xmath.h:850-880)
inline double dotr(const double* a, const double* b, int n, int sa = 1, int sb = 1) {
    if (n == 0) return 0.0;
    double t = a[(n - 1) * sa] * b[(n - 1) * sb];
    for (int k = n - 2; k >= 0; k--) t = a[k * sa] * b[k * sb] + t;
    return t;
}

// lower-triangular L with L L^T = M M^T (rows of M are the cell vectors,
// rotated so that the first lies on x and the second in the xy plane)
void rows_to_lower(const double M[3][3], double L[3][3]) {
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < i; j++) L[i][j] = (dotr(M[j], M[i], 3) - dotr(L[j], L[i], j)) / L[j][j];
        L[i][i] = sqrt(dotr(M[i], M[i], 3) - dotr(L[i], L[i], i));
        for (int j = i + 1; j < 3; j++) L[i][j] = 0.0;
    }
}

// B = H^-1 for lower-triangular H
void lower_inverse(const double H[3][3], double B[3][3]) {
    for (int i = 0; i < 3; i++) {
        B[i][i] = 1.0 / H[i][i];
        for (int d = 1; d <= i; d++) {
            int j = i - d;
            // sum over q = j..i-1 of B[q][j] H[i][q], right-nested
            B[i][j] = -B[i][i] * dotr(&B[j][j], &H[i][j], d, 3, 1);
        }
        for (int j = i + 1; j < 3; j++) B[i][j] = 0.0;
    }
}

// x = s H for lower-triangular H, as S2X on the packed columns
inline void s_to_x(const double H[3][3], const double* s, double* x) {
    x[0] = H[0][0] * s[0] + (H[1][0] * s[1] + H[2][0] * s[2]);
    x[1] = H[1][1] * s[1] + H[2][1] * s[2];
    x[2] = H[2][2] * s[2];
}

// s = x B, as X2S_NOCORR
inline void x_to_s(const double B[3][3], const double* x, double* s) {
    s[0] = B[0][0] * x[0] + (B[1][0] * x[1] + B[2][0] * x[2]);
    s[1] = B[1][1] * x[1] + B[2][1] * x[2];
    s[2] = B[2][2] * x[2];
}

// the reader's wrap: subtract 1 while s >= 1, then add 1 while s < 0 (the
// result can round to exactly 1.0 for tiny negative s)
inline double wrap_read(double s) {
    if (s >= 1.0) s -= floor(s);
    if (s < 0.0) s += ceil(-s);
    return s;
}

// the writer's wrap (X2S): add 1 while s < 0, then subtract 1 while s >= 1
inline double wrap_write(double s) {
    if (s < 0.0) s += ceil(-s);
    if (s >= 1.0) s -= floor(s);
    return s;
}

struct Header {
    int natoms = 0;
    bool empty = false;
    double A = 1.0, R = 1.0;
    int entry_count = 6;
    bool vel = true, ext = false;
    double H0[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double tr[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double eta[3][3] = {};
};

// header lines up to (not including) the first body line; returns its index
size_t read_header(const char* path, std::vector<std::string>& lines, Header& h) {
    const std::string file(path);
    size_t li = 0;
    for (; li < lines.size(); li++) {
        std::string& line = lines[li];
        int nw = normalise(line);
        if (nw == 0) continue;
        const char* c = line.c_str();
        int i, j, k;
        double t;
        if (sscanf(c, " Number of particles = %d ", &k) == 1) {
            if (k < 0) file_error("Number of particles in " + file + " file should be greater than 0");
            if (k == 0) h.empty = true;
            h.natoms = k;
            continue;
        }
        if (sscanf(c, " A = %lf ", &t) == 1) {
            if (t <= 0.0) file_error("A in " + file + " file should be greater than 0.0");
            h.A = t;
            continue;
        }
        if (line == ".NO_VELOCITY.") {
            // only before entry_count: afterwards the velocity columns stay
            if (!h.ext) {
                h.vel = false;
                h.ext = true;
            }
            continue;
        }
        if (sscanf(c, " entry_count = %d ", &k) == 1) {
            int minc = 3 + (h.vel ? 3 : 0);
            if (k < minc) file_error("entry_count in " + file + " should at least be equal to " + std::to_string(minc));
            h.entry_count = k;
            h.ext = true;
            continue;
        }
        if (sscanf(c, " R = %lf %*s ", &t) == 1) {
            h.R = t;
            continue;
        }
        if (sscanf(c, " auxiliary [ %d ] = %*s [ %*s ]", &i) == 1) {
            if (!h.ext) file_error("auxiliary [ ... ] = ... must come after entry_count = ... in " + file);
            int minc = 3 + (h.vel ? 3 : 0);
            if (i + minc + 1 > h.entry_count)
                file_error("wrong component in " + file + " file for auxiliary[" + std::to_string(i) + "]");
            continue;
        }
        if (sscanf(c, " Transform ( %d , %d ) = %lf ", &i, &j, &t) == 3) {
            if (i < 1 || i > 3 || j < 1 || j > 3)
                file_error("wrong component in " + file + " file for Transform(" + std::to_string(i) + "," +
                           std::to_string(j) + ")");
            h.tr[i - 1][j - 1] = t;
            continue;
        }
        if (sscanf(c, " H0 ( %d , %d ) = %lf  %*s", &i, &j, &t) == 3) {
            if (i < 1 || i > 3 || j < 1 || j > 3)
                file_error("wrong component in " + file + " file for H0(" + std::to_string(i) + "," +
                           std::to_string(j) + ")");
            h.H0[i - 1][j - 1] = t;
            continue;
        }
        if (sscanf(c, " eta ( %d , %d ) = %lf ", &i, &j, &t) == 3) {
            if (i < 1 || i > 3 || j < 1 || j > 3)
                file_error("wrong component in " + file + " file for eta(" + std::to_string(i) + "," +
                           std::to_string(j) + ")");
            h.eta[i - 1][j - 1] = t;
            continue;
        }
        if ((nw == 8 && !h.ext) || (nw == 1 && h.ext)) return li;  // first body line
        file_error("invalid line in " + file + " file: " + line);
    }
    if (!h.empty) file_error("file " + file + " ended unexpectedly");
    return li;
}

// the box of the header: (H0 Transform) [sqrt(1 + 2 eta)], made lower
// triangular, times A
void header_box(const char* path, Header& h, double H[3][3]) {
    double Hx[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double t = 0.0;
            for (int k = 0; k < 3; k++) t += h.H0[i][k] * h.tr[k][j];
            Hx[i][j] = t;
        }
    bool strained = false;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            if (h.eta[i][j] != 0.0) strained = true;
    if (strained) {
        double E[3][3], Es[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) E[i][j] = 2.0 * h.eta[i][j] + (i == j ? 1.0 : 0.0);
        if (!spd_sqrt3(E, Es)) file_error(std::string("eta in ") + path + " should be positive definite");
        double P[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double t = 0.0;
                for (int k = 0; k < 3; k++) t += Hx[i][k] * Es[k][j];
                P[i][j] = t;
            }
        memcpy(Hx, P, sizeof(P));
    }
    double L[3][3];
    rows_to_lower(Hx, L);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) H[i][j] = L[i][j] * h.A;
}

struct Elements {
    std::vector<double> masses;
    std::vector<std::string> names;
    // index of a name, added with this mass if new (Elements::add_type,
    // elements.cpp:93-114: an existing name keeps its first mass)
    uint8_t add(double mass, const char* name) {
        for (size_t i = 0; i < names.size(); i++)
            if (names[i] == name) return (uint8_t)i;
        if (names.size() == 255) file_error("cannot have more than 256 elements");
        masses.push_back(mass);
        names.emplace_back(name);
        return (uint8_t)(names.size() - 1);
    }
};

void read_body(const char* path, std::vector<std::string>& lines, size_t li, const Header& h, mappg_cfg& c) {
    const std::string file(path);
    Elements el;
    std::vector<double> s, sd;
    std::vector<uint8_t> elem;
    const size_t ncol = h.ext ? (size_t)h.entry_count : 8;
    const size_t first = h.ext ? 0 : 2;  // column of s_x
    bool mass_next_name = false, have_elem = false;
    double mass = 0.0;
    uint8_t ie = 0;
    int read = 0;
    for (; li < lines.size(); li++) {
        std::string& line = lines[li];
        normalise(line);
        const std::string text = line;  // words_of splits the line in place
        std::vector<const char*> w = words_of(line);
        size_t nw = w.size();
        if (nw == 0) continue;
        if (h.ext) {
            if (nw != 1 && nw != ncol) file_error("invalid line in " + file + " file: " + text);
            if (mass_next_name && nw != 1) file_error("expected chemical symbol of element after mass in " + file);
            if (nw == 1) {
                if (!mass_next_name) {
                    mass = atof(w[0]);
                    if (mass <= 0.0)
                        file_error(std::string("mass of ") + w[0] + " in " + file + " file should be greater than 0.0");
                    mass_next_name = true;
                } else {
                    ie = el.add(mass, w[0]);
                    mass_next_name = false;
                    have_elem = true;
                }
                continue;
            }
            if (!have_elem) file_error("line " + text + " in file " + file + " comes before any element was defined");
        } else {
            if (nw != 8) file_error("invalid line in " + file + " file: " + text);
            mass = atof(w[0]);
            if (mass <= 0.0)
                file_error(std::string("mass of ") + w[0] + " in " + file + " file should be greater than 0.0");
            ie = el.add(mass, w[1]);
        }
        double si[3];
        bool inside = true;
        for (int d = 0; d < 3; d++) {
            si[d] = atof(w[first + d]);
            if (!isfinite(si[d])) file_error("non-finite coordinate in " + file + " file: " + text);
            si[d] = wrap_read(si[d]);
            if (si[d] < 0.0 || si[d] >= 1.0) inside = false;
        }
        if (!inside) continue;  // not inserted: the count check below reports it
        s.insert(s.end(), si, si + 3);
        if (h.vel)
            for (int d = 0; d < 3; d++) sd.push_back(atof(w[first + 3 + d]));
        elem.push_back(ie);
        read++;
    }
    if (read != h.natoms)
        file_error("expected " + std::to_string(h.natoms) + " natms_lcl in " + file + " but read " +
                   std::to_string(read));
    c.natoms = read;
    c.has_vel = h.vel;
    c.masses = el.masses;
    c.names = el.names;
    c.elem.swap(elem);
    c.x.resize(3 * (size_t)read);
    for (int i = 0; i < read; i++) s_to_x(c.H, &s[3 * (size_t)i], &c.x[3 * (size_t)i]);
    if (h.vel) {
        // x_d = s_d (R H)
        double M[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) M[i][j] = h.R * c.H[i][j];
        c.v.resize(3 * (size_t)read);
        for (int i = 0; i < read; i++) s_to_x(M, &sd[3 * (size_t)i], &c.v[3 * (size_t)i]);
    }
}

}  // namespace
}  // namespace mappg

using namespace mappg;

extern "C" {

int mappg_cfg_read(const char* path, mappg_cfg** out) {
    return guard([&] {
        if (!path || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        std::vector<std::string> lines = read_lines(path);
        Header h;
        size_t li = read_header(path, lines, h);
        mappg_cfg* c = new mappg_cfg();
        try {
            header_box(path, h, c->H);
            if (li < lines.size())
                read_body(path, lines, li, h, *c);
            else
                c->natoms = 0;  // an empty configuration
        } catch (...) {
            delete c;
            throw;
        }
        *out = c;
    });
}

int mappg_cfg_info(const mappg_cfg* c, int* natoms, int* nelem, int* has_vel, double* H) {
    return guard([&] {
        if (!c) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (natoms) *natoms = c->natoms;
        if (nelem) *nelem = (int)c->names.size();
        if (has_vel) *has_vel = c->has_vel ? 1 : 0;
        if (H) memcpy(H, c->H, sizeof(c->H));
    });
}

int mappg_cfg_element(const mappg_cfg* c, int i, double* mass, char* name, int name_len) {
    return guard([&] {
        if (!c) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (i < 0 || i >= (int)c->names.size()) throw Error{MAPPG_ERR_ARG, "element index out of range"};
        if (mass) *mass = c->masses[i];
        if (name && name_len > 0) {
            if ((int)c->names[i].size() >= name_len) throw Error{MAPPG_ERR_ARG, "name buffer too short"};
            memcpy(name, c->names[i].c_str(), c->names[i].size() + 1);
        }
    });
}

int mappg_cfg_atoms(const mappg_cfg* c, double* x, double* x_d, unsigned char* elem) {
    return guard([&] {
        if (!c) throw Error{MAPPG_ERR_ARG, "null argument"};
        size_t n = (size_t)c->natoms;
        if (x && n) memcpy(x, c->x.data(), sizeof(double) * 3 * n);
        if (x_d && n) {
            if (!c->has_vel) throw Error{MAPPG_ERR_ARG, "the file has no velocities"};
            memcpy(x_d, c->v.data(), sizeof(double) * 3 * n);
        }
        if (elem && n) memcpy(elem, c->elem.data(), n);
    });
}

int mappg_cfg_destroy(mappg_cfg* c) {
    delete c;
    return MAPPG_OK;
}

int mappg_cfg_write(const char* path, int natoms, const double* H, const double* x, const unsigned char* elem,
                    int nelem, const double* masses, const char* const* names, int nvec,
                    const char* const* vec_names, const int* vec_dims, const double* const* vecs) {
    return guard([&] {
        if (!path || natoms < 0 || !H || (natoms && (!x || !elem)) || nelem < 0 || (nelem && (!masses || !names)) ||
            nvec < 0 || (nvec && (!vec_names || !vec_dims || !vecs)))
            throw Error{MAPPG_ERR_ARG, "null or negative argument"};
        double Hm[3][3], B[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Hm[i][j] = H[3 * i + j];
        if (Hm[0][1] != 0.0 || Hm[0][2] != 0.0 || Hm[1][2] != 0.0)
            throw Error{MAPPG_ERR_ARG, "the box must be lower triangular"};
        if (!(Hm[0][0] > 0.0 && Hm[1][1] > 0.0 && Hm[2][2] > 0.0))
            throw Error{MAPPG_ERR_ARG, "the box diagonal must be positive"};
        lower_inverse(Hm, B);
        int vel = -1;
        for (int k = 0; k < nvec; k++) {
            if (!vec_names[k] || vec_dims[k] < 1 || (natoms && !vecs[k]))
                throw Error{MAPPG_ERR_ARG, "invalid extra vector"};
            if (!strcmp(vec_names[k], "x_d")) {
                if (vec_dims[k] != 3) throw Error{MAPPG_ERR_ARG, "x_d must have 3 components"};
                vel = k;
            }
        }
        for (int i = 0; i < natoms; i++)
            if (elem[i] >= nelem) throw Error{MAPPG_ERR_ARG, "element index out of range"};
        FILE* fp = fopen(path, "w");
        if (!fp) throw Error{MAPPG_ERR_FILE, std::string("failed to open ") + path};
        int ncol = 3;
        for (int k = 0; k < nvec; k++) ncol += vec_dims[k];
        fprintf(fp, "Number of particles = %d\n", natoms);
        fprintf(fp, "A = %.16lf Angstrom (basic length-scale)\n", 1.0);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) fprintf(fp, "H0(%d,%d) = %.16lf A\n", i + 1, j + 1, Hm[i][j]);
        fprintf(fp, vel >= 0 ? "R = 1.0\n" : ".NO_VELOCITY.\n");
        fprintf(fp, "entry_count = %d\n", ncol);
        int aux = 0;
        for (int k = 0; k < nvec; k++) {
            if (k == vel) continue;
            for (int d = 0; d < vec_dims[k]; d++)
                fprintf(fp, "auxiliary[%d] = %s_%d [reduced unit]\n", aux++, vec_names[k], d);
        }
        int cur = -1;
        bool bad = false;
        for (int i = 0; i < natoms && !bad; i++) {
            if (elem[i] != cur) {
                cur = elem[i];
                fprintf(fp, "%lf\n", masses[cur]);
                fprintf(fp, "%s\n", names[cur]);
            }
            double s[3];
            const double* xi = x + 3 * (size_t)i;
            if (!isfinite(xi[0]) || !isfinite(xi[1]) || !isfinite(xi[2])) bad = true;
            x_to_s(B, xi, s);
            for (int d = 0; d < 3; d++) fprintf(fp, "%.16lf ", wrap_write(s[d]));
            for (int k = 0; k < nvec; k++) {
                const double* vk = vecs[k] + (size_t)vec_dims[k] * i;
                if (k == vel) {
                    double sd[3];
                    x_to_s(B, vk, sd);  // velocities in units of H per time, no wrap
                    for (int d = 0; d < 3; d++) fprintf(fp, "%.16lf ", sd[d]);
                } else {
                    for (int d = 0; d < vec_dims[k]; d++) fprintf(fp, "%.16lf ", vk[d]);
                }
            }
            fprintf(fp, "\n");
        }
        bool werr = ferror(fp) != 0;
        fclose(fp);
        if (bad) throw Error{MAPPG_ERR_NAN, "non-finite position"};
        if (werr) throw Error{MAPPG_ERR_FILE, std::string("failed to write ") + path};
    });
}

}  // extern "C"
