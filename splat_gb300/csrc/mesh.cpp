// mesh.cpp -- OBJ -> FTri, the reference's mesh_to_FTri (src/geo.jl:330-341)
// over the faces MeshIO loads.
//
// Each triangle corner keeps its own position, normal and uv (OBJ's v/vt/vn
// indices are per corner).  A polygon a b c d ... becomes the fan
// (a, b, c), (a, c, d), ... as process_face (src/geo.jl:289-304) and
// GeometryBasics' face decomposition do.  Record: cross(v1 - v2, v2 - v3),
// v1..v3, n1..n3, (u, v, 0) x 3 in binary32.  Numbers are read with strtof
// (correctly rounded decimal -> binary32, as Julia's parse(Float32, s)).
// Faces without normals get the unit face normal at every corner; faces
// without uvs get (0, 0, 0).
#include "mesh.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace splat {

namespace {

struct Corner {
    long v = 0, t = 0, n = 0;  // 1-based after resolution; 0 = absent
};

bool resolve(long idx, size_t count, long& out) {
    if (idx > 0) out = idx;
    else if (idx < 0) out = (long)count + idx + 1;
    else return false;
    return out >= 1 && (size_t)out <= count;
}

// "v", "v/t", "v//n", "v/t/n"
bool parse_corner(const char* tok, Corner& c) {
    char* end = nullptr;
    c.v = std::strtol(tok, &end, 10);
    if (end == tok) return false;
    if (*end == '/') {
        const char* p = end + 1;
        if (*p != '/') {
            c.t = std::strtol(p, &end, 10);
            if (end == p) return false;
        } else {
            end = const_cast<char*>(p);
        }
        if (*end == '/') {
            p = end + 1;
            c.n = std::strtol(p, &end, 10);
            if (end == p) return false;
        }
    }
    return *end == '\0';
}

}  // namespace

bool obj_to_ftri(const char* path, std::vector<splat_ftri_t>& out, std::string& err) {
    std::FILE* f = std::fopen(path, "r");
    if (!f) {
        err = std::string("cannot open ") + path;
        return false;
    }
    std::vector<float> V, N, T;  // xyz, xyz, uv
    std::vector<Corner> face;
    char line[4096];
    long lineno = 0;
    bool ok = true;
    while (ok && std::fgets(line, sizeof(line), f)) {
        ++lineno;
        char* save = nullptr;
        char* tok = strtok_r(line, " \t\r\n", &save);
        if (!tok || tok[0] == '#') continue;
        if (!std::strcmp(tok, "v") || !std::strcmp(tok, "vn") || !std::strcmp(tok, "vt")) {
            const bool is_t = tok[1] == 't';
            float xyz[3] = {0.f, 0.f, 0.f};
            int got = 0;
            for (int k = 0; k < 3; ++k) {
                char* s = strtok_r(nullptr, " \t\r\n", &save);
                if (!s) break;
                char* e = nullptr;
                xyz[k] = std::strtof(s, &e);
                if (e == s) {
                    ok = false;
                    break;
                }
                ++got;
            }
            if (!ok || got < (is_t ? 1 : 3)) {
                err = "bad vertex record at line " + std::to_string(lineno);
                ok = false;
                break;
            }
            std::vector<float>& dst = is_t ? T : (tok[1] == 'n' ? N : V);
            dst.push_back(xyz[0]);
            dst.push_back(xyz[1]);
            if (!is_t) dst.push_back(xyz[2]);
        } else if (!std::strcmp(tok, "f")) {
            face.clear();
            for (char* s = strtok_r(nullptr, " \t\r\n", &save); s; s = strtok_r(nullptr, " \t\r\n", &save)) {
                Corner c;
                if (!parse_corner(s, c) || !resolve(c.v, V.size() / 3, c.v) ||
                    (c.t && !resolve(c.t, T.size() / 2, c.t)) || (c.n && !resolve(c.n, N.size() / 3, c.n))) {
                    err = "bad face index at line " + std::to_string(lineno);
                    ok = false;
                    break;
                }
                face.push_back(c);
            }
            if (!ok) break;
            if (face.size() < 3) {
                err = "degenerate face at line " + std::to_string(lineno);
                ok = false;
                break;
            }
            for (size_t i = 2; i < face.size(); ++i) {
                const Corner cs[3] = {face[0], face[i - 1], face[i]};
                splat_ftri_t r;
                std::memset(&r, 0, sizeof(r));
                for (int k = 0; k < 3; ++k) {
                    for (int d = 0; d < 3; ++d) r.v[1 + k][d] = V[3 * (cs[k].v - 1) + d];
                    if (cs[k].t) {
                        r.v[7 + k][0] = T[2 * (cs[k].t - 1)];
                        r.v[7 + k][1] = T[2 * (cs[k].t - 1) + 1];
                    }
                }
                const float* v1 = r.v[1];
                const float* v2 = r.v[2];
                const float* v3 = r.v[3];
                const float a[3] = {v1[0] - v2[0], v1[1] - v2[1], v1[2] - v2[2]};
                const float b[3] = {v2[0] - v3[0], v2[1] - v3[1], v2[2] - v3[2]};
                r.v[0][0] = a[1] * b[2] - a[2] * b[1];
                r.v[0][1] = a[2] * b[0] - a[0] * b[2];
                r.v[0][2] = a[0] * b[1] - a[1] * b[0];
                const float* n = r.v[0];
                const float inv = 1.0f / std::sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]);
                for (int k = 0; k < 3; ++k)
                    for (int d = 0; d < 3; ++d)
                        r.v[4 + k][d] = cs[k].n ? N[3 * (cs[k].n - 1) + d] : n[d] * inv;
                out.push_back(r);
            }
        }
    }
    std::fclose(f);
    return ok;
}

}  // namespace splat
