// Dataset and variant file ingest of the reference's GPU prototype
// (src/gpu/import_dataset.cpp), behind the C ABI: host code only.
//
// Dataset files hold one point per line, "longitude,latitude[,value...]".
// importDataset (src/gpu/import_dataset.cpp:63-134) keeps
//   x = the latitude mapped to [0, 180]: ((90 - lat) / 90) * 90 for lat > 0,
//       ((-lat) / 90) * 90 + 90 otherwise (in FP64, operation by operation);
//   y = the longitude.
// Variant files hold "epsilon,minpts" per line; importDBScanInstances
// (src/gpu/import_dataset.cpp:232-262) sorts them with compareByEpsilon
// (import_dataset.cpp:41-49): epsilon descending, then minpts ascending.
//
// Fields are read like atof/atoi (leading blanks skipped, the longest numeric
// prefix taken, no prefix = 0).  Where the reference reads stale buffers (an
// empty field, a blank line) this reader skips blank lines and rejects empty
// fields; lines are not split at 399 characters.
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/vdbscan.h"

namespace {

// The comma-separated fields of one line (the newline removed).
std::vector<std::string> split_fields(const char* line) {
    std::vector<std::string> out;
    std::string cur;
    for (const char* p = line; *p && *p != '\n' && *p != '\r'; p++) {
        if (*p == ',') {
            out.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(*p);
        }
    }
    out.push_back(cur);
    return out;
}

bool blank(const char* line) {
    for (const char* p = line; *p; p++)
        if (!isspace((unsigned char)*p)) return false;
    return true;
}

// Reads the file line by line; fn(fields, line number) returns a VDB code.
template <class Fn>
int for_each_line(const char* path, Fn&& fn) {
    if (!path) return VDB_ERR_INVALID_ARG;
    FILE* f = fopen(path, "r");
    if (!f) return VDB_ERR_INVALID_ARG;
    std::string line;
    char buf[4096];
    int rc = VDB_OK;
    unsigned long lineno = 0;
    for (;;) {
        line.clear();
        bool got = false;
        while (fgets(buf, sizeof buf, f)) {
            got = true;
            line += buf;
            if (!line.empty() && line.back() == '\n') break;
        }
        if (!got) break;
        lineno++;
        if (blank(line.c_str())) continue;
        rc = fn(split_fields(line.c_str()), lineno);
        if (rc != VDB_OK) break;
    }
    fclose(f);
    return rc;
}

bool nonempty(const std::string& s) {
    for (char c : s)
        if (!isspace((unsigned char)c)) return true;
    return false;
}

// src/gpu/import_dataset.cpp:84-98
double map_latitude(double lat) {
    if (lat > 0.0) {
        const double deltaD = (90.0 - lat) / 90.0;
        return deltaD * 90.0;
    }
    const double deltaD = (-lat) / 90.0;
    return (deltaD * 90.0) + 90.0;
}

struct Variant {
    double eps;
    int minpts;
};

}  // namespace

extern "C" {

int vdb_import_dataset(const char* path, double* x, double* y, uint32_t cap, uint32_t* n) {
    if (!n) return VDB_ERR_INVALID_ARG;
    uint64_t count = 0;
    int rc = for_each_line(path, [&](const std::vector<std::string>& f, unsigned long) {
        if (f.size() < 2 || !nonempty(f[0]) || !nonempty(f[1])) return VDB_ERR_INVALID_ARG;
        if (count < cap) {
            const double lon = atof(f[0].c_str());
            const double lat = atof(f[1].c_str());
            if (x) x[count] = map_latitude(lat);
            if (y) y[count] = lon;
        }
        count++;
        return count > 0xffffffffull ? VDB_ERR_TOO_LARGE : VDB_OK;
    });
    *n = (uint32_t)std::min<uint64_t>(count, 0xffffffffull);
    if (rc != VDB_OK) return rc;
    if ((x || y) && count > cap) return VDB_ERR_CAPACITY;
    return VDB_OK;
}

int vdb_import_variants(const char* path, double* eps, uint32_t* minpts, uint32_t cap,
                        uint32_t* nv) {
    if (!nv) return VDB_ERR_INVALID_ARG;
    std::vector<Variant> vs;
    int rc = for_each_line(path, [&](const std::vector<std::string>& f, unsigned long) {
        if (f.size() < 2 || !nonempty(f[0]) || !nonempty(f[1])) return VDB_ERR_INVALID_ARG;
        Variant v{atof(f[0].c_str()), atoi(f[1].c_str())};
        if (v.minpts < 0) return VDB_ERR_INVALID_ARG;
        vs.push_back(v);
        return vs.size() > 0xffffffffull ? VDB_ERR_TOO_LARGE : VDB_OK;
    });
    *nv = (uint32_t)vs.size();
    if (rc != VDB_OK) return rc;
    // compareByEpsilon; NaN epsilons (unordered there) are put last
    std::stable_sort(vs.begin(), vs.end(), [](const Variant& a, const Variant& b) {
        const bool na = a.eps != a.eps, nb = b.eps != b.eps;
        if (na || nb) return !na && nb;
        if (a.eps == b.eps) return a.minpts < b.minpts;
        return a.eps > b.eps;
    });
    if ((eps || minpts) && vs.size() > cap) return VDB_ERR_CAPACITY;
    for (size_t i = 0; i < vs.size() && i < cap; i++) {
        if (eps) eps[i] = vs[i].eps;
        if (minpts) minpts[i] = (uint32_t)vs[i].minpts;
    }
    return VDB_OK;
}

}  // extern "C"
