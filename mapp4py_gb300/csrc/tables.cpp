// EAM table import and spline construction (host side, one-time).
//
// Readers follow ImportEAM (import_eam.h:68-901) and FileReader
// (import.cpp:92-240): lines are read whole, text after '#' is dropped,
// numbers may span lines but one line may not run past the end of a block
// ("file has extra arguments"), and a final line without a newline counts
// as the end of the file.  The spline builder is ImportEAM::interpolate
// (import_eam.cpp:62-83); the cutoff rule is set_cuttoff (import_eam.h:52-64).
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "internal.h"

namespace mappg {

namespace {

Error file_error(const std::string& path, const std::string& what) {
    return Error{MAPPG_ERR_FILE, path + ": " + what};
}

class LineReader {
   public:
    LineReader(const char* path) : path_(path) {
        f_ = fopen(path, "r");
        if (!f_) throw file_error(path_, "failed to open");
    }
    ~LineReader() {
        if (f_) fclose(f_);
    }
    // one line; false at end of file (a last line without '\n' is dropped)
    bool line(std::string& out) {
        if (finished_) return false;
        out.clear();
        int c;
        while ((c = fgetc(f_)) != EOF && c != '\n') out.push_back((char)c);
        if (c == EOF) {
            finished_ = true;
            return false;
        }
        return true;
    }
    // skip n lines; false when the file ends (FileReader::skip)
    bool skip(int n) {
        for (int i = 0; i < n && !finished_; i++) {
            int c;
            while ((c = fgetc(f_)) != EOF && c != '\n') {
            }
            if (c == EOF) finished_ = true;
        }
        if (!finished_) {
            int c = fgetc(f_);
            if (c == EOF)
                finished_ = true;
            else
                ungetc(c, f_);
        }
        return !finished_;
    }
    static std::vector<std::string> split(const std::string& s) {
        std::vector<std::string> out;
        size_t end = s.find('#');
        if (end == std::string::npos) end = s.size();
        size_t i = 0;
        while (i < end) {
            while (i < end && isspace((unsigned char)s[i])) i++;
            if (i >= end) break;
            size_t j = i;
            while (j < end && !isspace((unsigned char)s[j])) j++;
            out.push_back(s.substr(i, j - i));
            i = j;
        }
        return out;
    }
    // ImportEAM::read_double: n numbers, block must end at a line end
    void numbers(double* buf, size_t n) {
        size_t i = 0;
        std::string ln;
        while (i < n) {
            if (!line(ln)) throw file_error(path_, "file ended immaturely");
            auto a = split(ln);
            if (a.size() + i > n) throw file_error(path_, "file has extra arguments");
            for (auto& t : a) buf[i++] = atof(t.c_str());
        }
    }
    const std::string& path() const { return path_; }

   private:
    std::string path_;
    FILE* f_ = nullptr;
    bool finished_ = false;
};

// element header: map file elements to requested ones (elem_ref)
std::vector<int> map_elements(LineReader& r, int nreq, const char* const* req, HostTables& t,
                              std::vector<std::string>& file_names) {
    std::string ln;
    if (!r.line(ln)) throw file_error(r.path(), "file ended immaturely");
    auto a = LineReader::split(ln);
    if (a.size() < 2) throw file_error(r.path(), "invalid line: " + ln);
    size_t nref = a.size() - 1;
    file_names.assign(a.begin() + 1, a.end());
    std::vector<int> ref(nref, -1);
    if (nreq > 0) {
        std::vector<bool> found(nreq, false);
        for (size_t i = 0; i < nref; i++)
            for (int j = 0; j < nreq && ref[i] == -1; j++)
                if (file_names[i] == req[j]) {
                    found[j] = true;
                    ref[i] = j;
                }
        for (int j = 0; j < nreq; j++)
            if (!found[j])
                throw file_error(r.path(), std::string("file does not contain parameters for element ") + req[j]);
        t.names.assign(req, req + nreq);
    } else {
        for (size_t i = 0; i < nref; i++) ref[i] = (int)i;
        t.names = file_names;
    }
    return ref;
}

void read_grid_line(LineReader& r, size_t& nrho, double& drho, size_t& nr, double& dr) {
    std::string ln;
    if (!r.line(ln)) throw file_error(r.path(), "file ended immaturely");
    double rc;
    if (sscanf(ln.c_str(), " %zu %lf %zu %lf %lf", &nrho, &drho, &nr, &dr, &rc) != 5)
        throw file_error(r.path(), "invalid line: " + ln);
    if (nrho < 5) throw file_error(r.path(), "nrho should be larger than 5");
    if (nr < 5) throw file_error(r.path(), "nr should be larger than 5");
    if (drho <= 0.0) throw file_error(r.path(), "drho should be larger than 0.0");
    if (dr <= 0.0) throw file_error(r.path(), "dr should be larger than 0.0");
}

// ImportEAM::interpolate(type0*,size_t,type0,size_t)  import_eam.cpp:9-53:
// value of the local 5-point interpolant at knot k and fraction p
double interpolate_at(const double* arr, size_t n, double p, size_t k) {
    double c0 = arr[k], c1, c2, c3;
    if (k == 0) {
        c1 = arr[1] - arr[0];
        c2 = (-arr[0] + 2.0 * arr[1] - arr[2]) / 2.0;
        c3 = (arr[0] - 2.0 * arr[1] + arr[2]) / 2.0;
        return ((c3 * p + c2) * p + c1) * p + c0;
    } else if (k == 1) {
        c1 = 0.5 * (arr[2] - arr[0]);
        c2 = (11.0 * arr[0] - 28.0 * arr[1] + 24.0 * arr[2] - 8.0 * arr[3] + arr[4]) / 12.0;
        c3 = (-5.0 * arr[0] + 16.0 * arr[1] - 18.0 * arr[2] + 8.0 * arr[3] - arr[4]) / 12.0;
        return ((c3 * p + c2) * p + c1) * p + c0;
    } else if (k == n - 2) {
        c1 = 0.5 * (arr[n - 1] - arr[n - 3]);
        c2 = arr[n - 3] - 3.0 * arr[n - 2] + 2.0 * arr[n - 1];
        c3 = 0.5 * (-arr[n - 3] + 3.0 * arr[n - 2] - 2.0 * arr[n - 1]);
        return ((c3 * p + c2) * p + c1) * p + c0;
    } else if (k == n - 1) {
        c1 = arr[n - 1] - arr[n - 2];
        return c0 + c1 * p;
    }
    c1 = ((arr[k - 2] - arr[k + 2]) + 8.0 * (arr[k + 1] - arr[k - 1])) / 12.0;
    c2 = (-2.0 * arr[k - 2] + 15.0 * arr[k - 1] - 28.0 * arr[k] + 21.0 * arr[k + 1] - 6.0 * arr[k + 2]) / 12.0;
    c3 = (arr[k - 2] - 7.0 * arr[k - 1] + 16.0 * arr[k] - 17.0 * arr[k + 1] + 7.0 * arr[k + 2]) / 12.0;
    return ((c3 * p + c2) * p + c1) * p + c0;
}

}  // namespace

// ImportEAM::interpolate(size_t,type0,type0(*)[4])  import_eam.cpp:62-83
void interpolate4(size_t n, double (*s)[4]) {
    s[0][1] = s[1][0] - s[0][0];
    s[1][1] = 0.5 * (s[2][0] - s[0][0]);
    s[n - 2][1] = 0.5 * (s[n - 1][0] - s[n - 3][0]);
    s[n - 1][1] = s[n - 1][0] - s[n - 2][0];
    for (size_t i = 2; i < n - 2; i++)
        s[i][1] = ((s[i - 2][0] - s[i + 2][0]) + 8.0 * (s[i + 1][0] - s[i - 1][0])) / 12.0;
    for (size_t i = 0; i < n - 1; i++) {
        s[i][2] = 3.0 * (s[i + 1][0] - s[i][0]) - 2.0 * s[i][1] - s[i + 1][1];
        s[i][3] = s[i][1] + s[i + 1][1] - 2.0 * (s[i + 1][0] - s[i][0]);
    }
    s[n - 1][2] = 0.0;
    s[n - 1][3] = 0.0;
}

void HostTables::alloc(int ne, int nr_, int nrho_, double dr_, double drho_) {
    if (ne < 1 || ne > kMaxElem) throw Error{MAPPG_ERR_ARG, "this engine supports 1.." + std::to_string(kMaxElem) + " elements"};
    nelem = ne;
    nr = nr_;
    nrho = nrho_;
    dr = dr_;
    drho = drho_;
    F.assign((size_t)ne * nrho * 4, 0.0);
    rho.assign((size_t)ne * ne * nr * 4, 0.0);
    rphi.assign((size_t)ne * ne * nr * 4, 0.0);
    cut.assign((size_t)ne * ne, 0.0);
}

// splines for every table, mirror of rphi[i][j] into [j][i], then the
// cutoff: last knot where rphi, rho[i][j] and rho[j][i] are not all zero
void HostTables::finish_splines(bool per_pair_rho) {
    for (int i = 0; i < nelem; i++) interpolate4((size_t)nrho, (double(*)[4])F_at(i));
    for (int i = 0; i < nelem; i++) {
        if (per_pair_rho) {
            for (int j = 0; j < nelem; j++) interpolate4((size_t)nr, (double(*)[4])rho_at(i, j));
        } else {
            interpolate4((size_t)nr, (double(*)[4])rho_at(i, 0));
            for (int j = 1; j < nelem; j++) memcpy(rho_at(i, j), rho_at(i, 0), sizeof(double) * 4 * nr);
        }
    }
    for (int i = 0; i < nelem; i++)
        for (int j = 0; j <= i; j++) {
            interpolate4((size_t)nr, (double(*)[4])rphi_at(i, j));
            if (i != j) memcpy(rphi_at(j, i), rphi_at(i, j), sizeof(double) * 4 * nr);
        }
    for (int i = 0; i < nelem; i++)
        for (int j = 0; j < i + 1; j++) {
            size_t n_ = (size_t)nr - 1;
            while ((rphi_at(i, j)[4 * n_] == 0.0 && rho_at(i, j)[4 * n_] == 0.0 && rho_at(j, i)[4 * n_] == 0.0) && n_ >= 1)
                n_--;
            cut[i * nelem + j] = cut[j * nelem + i] = (double)n_ * dr;
        }
}

// ImportEAM::setfl  import_eam.h:348-613
void read_setfl(const char* path, int nreq, const char* const* req, HostTables& t) {
    LineReader r(path);
    if (!r.skip(3)) throw file_error(path, "file ended immaturely");
    std::vector<std::string> fnames;
    std::vector<int> ref = map_elements(r, nreq, req, t, fnames);
    size_t nref = ref.size();
    int ne = (int)t.names.size();
    size_t nrho, nr;
    double drho, dr;
    read_grid_line(r, nrho, drho, nr, dr);
    t.alloc(ne, (int)nr, (int)nrho, dr, drho);
    std::vector<double> buf(std::max(nr + nrho, nref * (nref + 1) / 2 * nr));
    for (size_t i = 0; i < nref; i++) {
        if (!r.skip(1)) throw file_error(path, "file ended immaturely");
        r.numbers(buf.data(), nrho + nr);
        int ie = ref[i];
        if (ie == -1) continue;
        for (size_t k = 0; k < nrho; k++) t.F_at(ie)[4 * k] = buf[k];
        for (size_t k = 0; k < nr; k++) t.rho_at(ie, 0)[4 * k] = buf[k + nrho];
    }
    r.numbers(buf.data(), nref * (nref + 1) / 2 * nr);
    size_t ipos = 0;
    for (size_t i = 0; i < nref; i++)
        for (size_t j = 0; j < i + 1; j++) {
            int ie = ref[i], je = ref[j];
            if (ie == -1 || je == -1) {
                ipos += nr;
                continue;
            }
            double* dst = t.rphi_at(std::max(ie, je), std::min(ie, je));
            for (size_t k = 0; k < nr; k++) dst[4 * k] = buf[ipos++];
        }
    t.finish_splines(false);
}

// ImportEAM::fs  import_eam.h:617-901: per element F then rho[i][j] for
// every j, then the symmetric r*phi block
void read_fs(const char* path, int nreq, const char* const* req, HostTables& t) {
    LineReader r(path);
    if (!r.skip(3)) throw file_error(path, "file ended immaturely");
    std::vector<std::string> fnames;
    std::vector<int> ref = map_elements(r, nreq, req, t, fnames);
    size_t nref = ref.size();
    int ne = (int)t.names.size();
    size_t nrho, nr;
    double drho, dr;
    read_grid_line(r, nrho, drho, nr, dr);
    t.alloc(ne, (int)nr, (int)nrho, dr, drho);
    std::vector<double> buf(std::max(nrho + nr * nref, nref * (nref + 1) / 2 * nr));
    for (size_t i = 0; i < nref; i++) {
        if (!r.skip(1)) throw file_error(path, "file ended immaturely");
        r.numbers(buf.data(), nrho + nr * nref);
        int ie = ref[i];
        if (ie == -1) continue;
        for (size_t k = 0; k < nrho; k++) t.F_at(ie)[4 * k] = buf[k];
        size_t ipos = nrho;
        for (size_t j = 0; j < nref; j++) {
            int je = ref[j];
            if (je == -1) {
                ipos += nr;
                continue;
            }
            for (size_t k = 0; k < nr; k++) t.rho_at(ie, je)[4 * k] = buf[ipos++];
        }
    }
    r.numbers(buf.data(), nref * (nref + 1) / 2 * nr);
    size_t ipos = 0;
    for (size_t i = 0; i < nref; i++)
        for (size_t j = 0; j < i + 1; j++) {
            int ie = ref[i], je = ref[j];
            if (ie == -1 || je == -1) {
                ipos += nr;
                continue;
            }
            double* dst = t.rphi_at(std::max(ie, je), std::min(ie, je));
            for (size_t k = 0; k < nr; k++) dst[4 * k] = buf[ipos++];
        }
    t.finish_splines(true);
}

// ImportEAM::funcfl  import_eam.h:68-346: one file per element, resampled
// onto the coarsest grid; r*phi_ij = 27.2*0.529*Z_i*Z_j.  The reference
// evaluates Z at knot index k rather than at the interval index (lines
// 290,298); that choice is kept.
void read_funcfl(int nfiles, const char* const* paths, HostTables& t) {
    if (nfiles < 1) throw Error{MAPPG_ERR_ARG, "ff_eam_funcfl needs at least one file"};
    std::vector<size_t> nrs(nfiles), nrhos(nfiles);
    std::vector<double> drs(nfiles), drhos(nfiles);
    std::vector<std::vector<double>> Fk(nfiles), Zk(nfiles), Rk(nfiles);
    for (int i = 0; i < nfiles; i++) {
        LineReader r(paths[i]);
        if (!r.skip(2)) throw file_error(paths[i], "file ended immaturely");
        read_grid_line(r, nrhos[i], drhos[i], nrs[i], drs[i]);
        std::vector<double> buf(nrhos[i] + 2 * nrs[i]);
        r.numbers(buf.data(), buf.size());
        Fk[i].assign(buf.begin(), buf.begin() + nrhos[i]);
        Zk[i].assign(buf.begin() + nrhos[i], buf.begin() + nrhos[i] + nrs[i]);
        Rk[i].assign(buf.begin() + nrhos[i] + nrs[i], buf.end());
    }
    double maxr = 0, maxrho = 0, maxdr = 0, maxdrho = 0;
    for (int i = 0; i < nfiles; i++) {
        maxr = std::max(maxr, (double)(nrs[i] - 1) * drs[i]);
        maxrho = std::max(maxrho, (double)(nrhos[i] - 1) * drhos[i]);
        maxdr = std::max(maxdr, drs[i]);
        maxdrho = std::max(maxdrho, drhos[i]);
    }
    size_t nr = (size_t)(maxr / maxdr + 0.5), nrho = (size_t)(maxrho / maxdrho + 0.5);
    for (int i = 0; i < nfiles; i++)
        if (nr > nrs[i]) throw Error{MAPPG_ERR_FILE, std::string(paths[i]) + ": its r grid is shorter than the common grid"};
    t.alloc(nfiles, (int)nr, (int)nrho, maxdr, maxdrho);
    t.names.assign(nfiles, "");
    auto frac = [](double x, double d, size_t n, size_t& l) {
        double p = x / d;
        l = (size_t)p;
        l = std::min(l, n - 2);
        p -= (double)l;
        return std::min(p, 1.0);
    };
    size_t l;
    for (int i = 0; i < nfiles; i++)
        for (int j = 0; j < i + 1; j++)
            for (size_t k = 0; k < nr; k++) {
                double rr = (double)k * maxdr;
                double p0 = frac(rr, drs[i], nrs[i], l);
                double z0 = interpolate_at(Zk[i].data(), nrs[i], p0, k);
                double p1 = frac(rr, drs[j], nrs[j], l);
                double z1 = interpolate_at(Zk[j].data(), nrs[j], p1, k);
                t.rphi_at(i, j)[4 * k] = 27.2 * 0.529 * z0 * z1;
            }
    for (int i = 0; i < nfiles; i++)
        for (size_t k = 0; k < nr; k++) {
            double rr = (double)k * maxdr;
            double p = frac(rr, drs[i], nrs[i], l);
            t.rho_at(i, 0)[4 * k] = interpolate_at(Rk[i].data(), nrs[i], p, l);
        }
    for (int i = 0; i < nfiles; i++)
        for (size_t k = 0; k < nrho; k++) {
            double rh = (double)k * maxdrho;
            double p = frac(rh, drhos[i], nrhos[i], l);
            t.F_at(i)[4 * k] = interpolate_at(Fk[i].data(), nrhos[i], p, l);
        }
    t.finish_splines(false);
}

}  // namespace mappg
