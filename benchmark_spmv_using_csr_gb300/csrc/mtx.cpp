// mtx.cpp -- Matrix Market coordinate files to CSR (the loader of spmv_cuda/main.cu:570-733).
//
// The file is read whole and tokenised in one pass; the entries go to a triplet list, then a
// stable counting sort by row builds the CSR exactly as the reference's does (row counts, an
// exclusive scan, placement in file order with each mirrored entry placed right after its
// source entry).
#include <cctype>
#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/spmv_mtx.h"

struct bhsp_mtx {
    bhsp_mtx_info info;
    std::vector<int> row_ptr;
    std::vector<int> col;
    std::vector<double> val;
};

namespace {

bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f';
}

// One line of the buffer: [begin, end) without the newline; pos moves past it.
bool next_line(const std::string& buf, size_t& pos, std::string& line) {
    if (pos >= buf.size()) return false;
    size_t e = buf.find('\n', pos);
    if (e == std::string::npos) e = buf.size();
    line.assign(buf, pos, e - pos);
    pos = e < buf.size() ? e + 1 : e;
    return true;
}

std::vector<std::string> tokens(const std::string& line) {
    std::vector<std::string> t;
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && is_space(line[i])) ++i;
        size_t j = i;
        while (j < line.size() && !is_space(line[j])) ++j;
        if (j > i) t.emplace_back(line, i, j - i);
        i = j;
    }
    return t;
}

std::string lower(std::string s) {
    for (char& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

// mm_read_banner (mmio.h:249-330): 5 tokens, "%%MatrixMarket" prefix, then matrix /
// coordinate|array / real|complex|pattern|integer / general|symmetric|hermitian|skew-symmetric.
int parse_banner(const std::string& line, bool& array, int& field, int& symmetry, bool& complex) {
    const std::vector<std::string> t = tokens(line);
    if (t.size() < 5) return BHSP_MTX_BAD_BANNER;
    if (t[0].compare(0, 14, "%%MatrixMarket") != 0) return BHSP_MTX_BAD_BANNER;
    if (lower(t[1]) != "matrix") return BHSP_MTX_BAD_BANNER;
    const std::string crd = lower(t[2]), data = lower(t[3]), sym = lower(t[4]);
    if (crd == "coordinate")
        array = false;
    else if (crd == "array")
        array = true;
    else
        return BHSP_MTX_BAD_BANNER;
    complex = false;
    if (data == "real")
        field = 0;
    else if (data == "integer")
        field = 1;
    else if (data == "pattern")
        field = 2;
    else if (data == "complex")
        complex = true;
    else
        return BHSP_MTX_BAD_BANNER;
    if (sym == "general")
        symmetry = 0;
    else if (sym == "symmetric")
        symmetry = 1;
    else if (sym == "hermitian")
        symmetry = 2;
    else if (sym == "skew-symmetric")
        symmetry = 3;
    else
        return BHSP_MTX_BAD_BANNER;
    return BHSP_MTX_OK;
}

struct Cursor {
    const char* p;
    const char* end;
    void skip() {
        while (p < end && is_space(*p)) ++p;
    }
    bool read_long(long long& v) {
        skip();
        if (p >= end) return false;
        char* q = nullptr;
        errno = 0;
        v = std::strtoll(p, &q, 10);
        if (q == p || errno == ERANGE) return false;
        p = q;
        return true;
    }
    bool read_double(double& v) {
        skip();
        if (p >= end) return false;
        char* q = nullptr;
        v = std::strtod(p, &q);
        if (q == p) return false;
        p = q;
        return true;
    }
};

int load(const char* path, bhsp_mtx* a) {
    std::FILE* f = std::fopen(path, "rb");
    if (f == nullptr) return BHSP_MTX_OPEN_FAILED;
    std::string buf;
    {
        char chunk[1 << 16];
        size_t k;
        while ((k = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.append(chunk, k);
        std::fclose(f);
    }
    size_t pos = 0;
    std::string line;
    if (!next_line(buf, pos, line)) return BHSP_MTX_BAD_BANNER;
    bool array = false, complex = false;
    int field = 0, symmetry = 0;
    int rc = parse_banner(line, array, field, symmetry, complex);
    if (rc != BHSP_MTX_OK) return rc;
    if (complex) return BHSP_MTX_COMPLEX;
    if (array) return BHSP_MTX_UNSUPPORTED;

    // mm_read_mtx_crd_size (mmio.h:334-357): skip '%' lines, then the first line with 3 ints
    long long M = 0, N = 0, NZ = 0;
    for (;;) {
        if (!next_line(buf, pos, line)) return BHSP_MTX_BAD_SIZE;
        if (!line.empty() && line[0] == '%') continue;
        const std::vector<std::string> t = tokens(line);
        if (t.empty()) continue;  // blank line: the size comes later
        if (t.size() < 3) return BHSP_MTX_BAD_SIZE;
        char* q = nullptr;
        M = std::strtoll(t[0].c_str(), &q, 10);
        if (*q) return BHSP_MTX_BAD_SIZE;
        N = std::strtoll(t[1].c_str(), &q, 10);
        if (*q) return BHSP_MTX_BAD_SIZE;
        NZ = std::strtoll(t[2].c_str(), &q, 10);
        if (*q) return BHSP_MTX_BAD_SIZE;
        break;
    }
    if (M < 0 || N < 0 || NZ < 0 || M > INT_MAX - 1 || N > INT_MAX || NZ > INT_MAX)
        return BHSP_MTX_BAD_SIZE;
    const int m = (int)M, n = (int)N, nzf = (int)NZ;
    const bool mirror = symmetry == 1 || symmetry == 2;

    std::vector<int> ri, ci;
    std::vector<double> vi;
    try {
        ri.resize(nzf);
        ci.resize(nzf);
        vi.resize(nzf);
    } catch (const std::bad_alloc&) {
        return BHSP_MTX_NO_MEMORY;
    }
    Cursor c{buf.data() + pos, buf.data() + buf.size()};
    for (int e = 0; e < nzf; ++e) {
        long long i = 0, j = 0;
        if (!c.read_long(i) || !c.read_long(j)) return BHSP_MTX_BAD_ENTRY;
        double v = 1.0;  // pattern
        if (field == 0) {
            if (!c.read_double(v)) return BHSP_MTX_BAD_ENTRY;
        } else if (field == 1) {
            long long iv = 0;
            if (!c.read_long(iv) || iv < INT_MIN || iv > INT_MAX) return BHSP_MTX_BAD_ENTRY;
            v = (double)(int)iv;
        }
        if (i < 1 || i > m || j < 1 || j > n) return BHSP_MTX_BAD_ENTRY;
        if (mirror && i != j && (j > m || i > n)) return BHSP_MTX_BAD_ENTRY;
        ri[e] = (int)(i - 1);
        ci[e] = (int)(j - 1);
        vi[e] = v;
    }

    // counting sort by row (main.cu:618-716)
    std::vector<long long> cnt((size_t)m + 1, 0);
    for (int e = 0; e < nzf; ++e) {
        ++cnt[ri[e]];
        if (mirror && ri[e] != ci[e]) ++cnt[ci[e]];
    }
    long long run = 0;
    for (int r = 0; r <= m; ++r) {
        const long long k = cnt[r];
        cnt[r] = run;
        run += k;
    }
    if (run > INT_MAX) return BHSP_MTX_TOO_LARGE;
    const int nnz = (int)run;
    try {
        a->row_ptr.resize((size_t)m + 1);
        a->col.resize(nnz);
        a->val.resize(nnz);
    } catch (const std::bad_alloc&) {
        return BHSP_MTX_NO_MEMORY;
    }
    for (int r = 0; r <= m; ++r) a->row_ptr[r] = (int)cnt[r];
    for (int e = 0; e < nzf; ++e) {
        const long long o = cnt[ri[e]]++;
        a->col[o] = ci[e];
        a->val[o] = vi[e];
        if (mirror && ri[e] != ci[e]) {
            const long long o2 = cnt[ci[e]]++;
            a->col[o2] = ri[e];
            a->val[o2] = vi[e];
        }
    }
    a->info.m = m;
    a->info.n = n;
    a->info.nnz_file = nzf;
    a->info.nnz = nnz;
    a->info.field = field;
    a->info.symmetry = symmetry;
    return BHSP_MTX_OK;
}

}  // namespace

extern "C" int bhsp_mtx_load(const char* path, bhsp_mtx** out) {
    if (out == nullptr) return BHSP_MTX_OPEN_FAILED;
    *out = nullptr;
    if (path == nullptr) return BHSP_MTX_OPEN_FAILED;
    bhsp_mtx* a = new (std::nothrow) bhsp_mtx();
    if (a == nullptr) return BHSP_MTX_NO_MEMORY;
    int rc;
    try {
        rc = load(path, a);
    } catch (const std::bad_alloc&) {
        rc = BHSP_MTX_NO_MEMORY;
    }
    if (rc != BHSP_MTX_OK) {
        delete a;
        return rc;
    }
    *out = a;
    return BHSP_MTX_OK;
}

extern "C" int bhsp_mtx_get_info(const bhsp_mtx* a, bhsp_mtx_info* info) {
    if (a == nullptr || info == nullptr) return BHSP_MTX_BAD_ENTRY;
    *info = a->info;
    return BHSP_MTX_OK;
}

extern "C" const int* bhsp_mtx_row_ptr(const bhsp_mtx* a) { return a ? a->row_ptr.data() : nullptr; }
extern "C" const int* bhsp_mtx_col_idx(const bhsp_mtx* a) { return a ? a->col.data() : nullptr; }
extern "C" const double* bhsp_mtx_val(const bhsp_mtx* a) { return a ? a->val.data() : nullptr; }
extern "C" void bhsp_mtx_free(bhsp_mtx* a) { delete a; }
