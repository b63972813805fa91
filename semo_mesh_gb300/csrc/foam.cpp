// OpenFOAM polyMesh reader: the file parsing of SEMO_Mesh_Load::OpenFoam
// (src/load/loadOpenFoam.cpp:16-350), ASCII lists as SEMO reads them.
//
//   points     "(x y z)" per entry, each coordinate parsed to long double
//              and rounded to double (SEMO reads them with stold)
//   faces      "n(p0 ... pn-1)" per face, possibly over several lines
//   owner      one label per face
//   neighbour  one label per internal face (the list ends at ')' or at a
//              negative label)
//   boundary   name { ... nFaces N; startFace S; ... } per patch
// Each list starts after the first line whose first character is '(' and
// ends at the first line starting with ')', which skips the FoamFile header
// and the count line as SEMO's loop does.  What SEMO does after reading
// (loadOpenFoam.cpp:356-374: cells, face types, lists, cellsGlobal) is the
// mesh upload's job.  Host code only: nothing here touches the GPU.
#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "semo_internal.h"

namespace {

using semo::Error;

thread_local std::string g_foam_err;

struct FoamMesh {
    std::vector<double> pts;
    std::vector<int32_t> fptr{0}, fpts, own, nei;
    std::vector<std::string> names;
    std::vector<int32_t> pstart, psize;
    int64_t n_cells = 0;
};

// the lines of a list body: after the first line starting with '(' up to
// (not including) the first line starting with ')'
std::vector<std::string> body(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw Error(SEMO_ERR_ARGUMENT, "cannot open " + path);
    std::vector<std::string> out;
    std::string line;
    bool started = false;
    while (std::getline(in, line)) {
        if (!started) {
            if (!line.empty() && line[0] == '(') started = true;
            continue;
        }
        if (!line.empty() && line[0] == ')') return out;
        out.push_back(line);
    }
    if (!started) throw Error(SEMO_ERR_MESH, "no list in " + path);
    throw Error(SEMO_ERR_MESH, "list not closed in " + path);
}

// every integer of a text, '(' and ')' taken as separators
std::vector<long long> labels(const std::vector<std::string>& lines) {
    std::vector<long long> v;
    for (const std::string& l : lines) {
        const char* p = l.c_str();
        while (*p) {
            if (*p == '-' || std::isdigit((unsigned char)*p)) {
                char* e = nullptr;
                v.push_back(std::strtoll(p, &e, 10));
                p = e;
            } else {
                ++p;
            }
        }
    }
    return v;
}

void read_points(const std::string& dir, FoamMesh& m) {
    for (const std::string& l : body(dir + "/points")) {
        std::string t = l;
        for (char& ch : t) if (ch == '(' || ch == ')') ch = ' ';
        const char* p = t.c_str();
        int k = 0;
        while (true) {
            while (*p && std::isspace((unsigned char)*p)) ++p;
            if (!*p) break;
            char* e = nullptr;
            const long double x = std::strtold(p, &e);
            if (e == p) throw Error(SEMO_ERR_MESH, "bad number in points: " + l);
            m.pts.push_back((double)x);
            p = e;
            ++k;
        }
        if (k != 0 && k != 3) throw Error(SEMO_ERR_MESH, "a point needs three coordinates: " + l);
    }
}

void read_faces(const std::string& dir, FoamMesh& m) {
    const std::vector<long long> v = labels(body(dir + "/faces"));
    size_t i = 0;
    while (i < v.size()) {
        const long long n = v[i++];
        if (n < 3 || i + (size_t)n > v.size()) throw Error(SEMO_ERR_MESH, "truncated or degenerate face list");
        for (long long k = 0; k < n; ++k) m.fpts.push_back((int32_t)v[i++]);
        m.fptr.push_back((int32_t)m.fpts.size());
    }
}

void read_owner_neighbour(const std::string& dir, FoamMesh& m) {
    for (long long x : labels(body(dir + "/owner"))) m.own.push_back((int32_t)x);
    for (long long x : labels(body(dir + "/neighbour"))) {
        if (x < 0) break;
        m.nei.push_back((int32_t)x);
    }
    long long mx = -1;
    for (int32_t x : m.own) mx = std::max<long long>(mx, x);
    for (int32_t x : m.nei) mx = std::max<long long>(mx, x);
    m.n_cells = mx + 1;
}

void read_boundary(const std::string& dir, FoamMesh& m) {
    const std::vector<std::string> lines = body(dir + "/boundary");
    std::string prev;
    bool inside = false;
    long long nf = -1, sf = -1;
    for (const std::string& raw : lines) {
        std::string l = raw;
        const size_t a = l.find_first_not_of(" \t\r"), b = l.find_last_not_of(" \t\r");
        l = (a == std::string::npos) ? std::string() : l.substr(a, b - a + 1);
        if (!inside) {
            if (l.find('{') != std::string::npos) {
                std::string name = l.substr(0, l.find('{'));
                const size_t c = name.find_last_not_of(" \t");
                name = (c == std::string::npos) ? prev : name.substr(0, c + 1);
                m.names.push_back(name);
                inside = true;
                nf = sf = -1;
            } else if (!l.empty()) {
                prev = l;
            }
            continue;
        }
        if (l.find('}') != std::string::npos) {
            if (nf < 0 || sf < 0) throw Error(SEMO_ERR_MESH, "patch " + m.names.back() + " lacks nFaces or startFace");
            m.psize.push_back((int32_t)nf);
            m.pstart.push_back((int32_t)sf);
            inside = false;
            continue;
        }
        std::istringstream iss(l);
        std::string key;
        long long val = 0;
        iss >> key;
        if (key == "nFaces" && (iss >> val)) nf = val;
        if (key == "startFace" && (iss >> val)) sf = val;
    }
    if (inside) throw Error(SEMO_ERR_MESH, "boundary dictionary not closed");
}

void read_all(const char* dir, FoamMesh& m) {
    if (!dir) throw Error(SEMO_ERR_ARGUMENT, "null directory");
    const std::string d(dir);
    read_points(d, m);
    read_faces(d, m);
    read_owner_neighbour(d, m);
    read_boundary(d, m);
    const size_t nf = m.fptr.size() - 1;
    if (m.own.size() != nf) throw Error(SEMO_ERR_MESH, "owner list and face list differ in length");
    if (m.nei.size() > nf) throw Error(SEMO_ERR_MESH, "more neighbours than faces");
}

template <class F>
semo_status free_guarded(F&& f) {
    try {
        g_foam_err.clear();
        f();
        return SEMO_OK;
    } catch (const Error& e) {
        g_foam_err = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        g_foam_err = "host allocation failed";
        return SEMO_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        g_foam_err = e.what();
        return SEMO_ERR_MESH;
    }
}

}  // namespace

extern "C" {

const char* semo_foam_last_error(void) { return g_foam_err.c_str(); }

semo_status semo_foam_sizes(const char* dir, int64_t* out6) {
    return free_guarded([&] {
        if (!out6) throw Error(SEMO_ERR_ARGUMENT, "null output");
        FoamMesh m;
        read_all(dir, m);
        out6[0] = (int64_t)(m.pts.size() / 3);
        out6[1] = (int64_t)(m.fptr.size() - 1);
        out6[2] = (int64_t)m.nei.size();
        out6[3] = m.n_cells;
        out6[4] = (int64_t)m.fpts.size();
        out6[5] = (int64_t)m.names.size();
    });
}

semo_status semo_foam_read(const char* dir, double* points, int32_t* face_ptr, int32_t* face_pts, int32_t* owner,
                           int32_t* neighbour, int32_t* patch_start, int32_t* patch_size, char* patch_names) {
    return free_guarded([&] {
        FoamMesh m;
        read_all(dir, m);
        if (points) std::memcpy(points, m.pts.data(), sizeof(double) * m.pts.size());
        if (face_ptr) std::memcpy(face_ptr, m.fptr.data(), sizeof(int32_t) * m.fptr.size());
        if (face_pts) std::memcpy(face_pts, m.fpts.data(), sizeof(int32_t) * m.fpts.size());
        if (owner) std::memcpy(owner, m.own.data(), sizeof(int32_t) * m.own.size());
        if (neighbour) std::memcpy(neighbour, m.nei.data(), sizeof(int32_t) * m.nei.size());
        if (patch_start) std::memcpy(patch_start, m.pstart.data(), sizeof(int32_t) * m.pstart.size());
        if (patch_size) std::memcpy(patch_size, m.psize.data(), sizeof(int32_t) * m.psize.size());
        if (patch_names)
            for (size_t p = 0; p < m.names.size(); ++p) {
                char* dst = patch_names + 64 * p;
                std::memset(dst, 0, 64);
                std::strncpy(dst, m.names[p].c_str(), 63);
            }
    });
}

semo_status semo_mesh_load_foam(semo_ctx* ctx, const char* dir) {
    if (!ctx) return SEMO_ERR_ARGUMENT;
    FoamMesh m;
    const semo_status st = free_guarded([&] { read_all(dir, m); });
    if (st != SEMO_OK) {
        ctx->err = g_foam_err;
        return st;
    }
    return semo_mesh_upload(ctx, (int)(m.pts.size() / 3), m.pts.data(), (int)(m.fptr.size() - 1), (int)m.nei.size(),
                            (int)m.n_cells, m.fptr.data(), m.fpts.data(), m.own.data(), m.nei.data(),
                            (int)m.names.size(), m.pstart.data(), m.psize.data());
}

}  // extern "C"
