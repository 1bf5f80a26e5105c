// Triangle-mesh OBJ reading and writing (read_obj / write_obj, read_obj.cpp:8-63).
//
// The reference reader treats every line that starts with 'v' as a vertex and parses face
// records as three plain integers, so a file with normals ("vn"), texture coordinates ("vt") or
// "f a/b/c" face records is rejected. This reader takes "v" records only (x y z, an optional w
// ignored), skips "vn", "vt", "vp", comments and grouping / material records, reads the vertex
// index of "a", "a/b", "a//c" and "a/b/c" face tokens, and resolves negative (relative) indices
// as the OBJ format defines them. Faces with other than three vertices are an error, as in the
// reference. The writer prints full-precision vertices (17 significant digits, so that a write /
// read round trip is exact) and 1-based faces.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ac3d.h"

namespace {

struct ObjMesh {
  std::vector<double> P;
  std::vector<int32_t> E;
  std::string err;
};

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f'; }

// Reads the whole file; returns false with a message on malformed input.
bool parse_obj(const char* path, ObjMesh& m) {
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    m.err = std::string("cannot open ") + path;
    return false;
  }
  std::string line;
  std::vector<char> buf(1 << 16);
  bool ok = true;
  long lineno = 0;
  auto fail = [&](const char* what) {
    m.err = std::string(what) + " at line " + std::to_string(lineno);
    ok = false;
  };
  while (ok) {
    line.clear();
    bool got = false;
    while (std::fgets(buf.data(), (int)buf.size(), f)) {
      got = true;
      line += buf.data();
      if (!line.empty() && line.back() == '\n') break;
    }
    if (!got) break;
    lineno++;
    const char* s = line.c_str();
    while (*s && is_space(*s)) s++;
    if (s[0] == 'v' && is_space(s[1])) {
      const char* q = s + 1;
      double xyz[3];
      for (int d = 0; d < 3; d++) {
        char* end = nullptr;
        errno = 0;
        xyz[d] = std::strtod(q, &end);
        if (end == q || errno == ERANGE) {
          fail("invalid vertex specification");
          break;
        }
        q = end;
      }
      if (!ok) break;
      m.P.insert(m.P.end(), xyz, xyz + 3);
    } else if (s[0] == 'f' && is_space(s[1])) {
      const char* q = s + 1;
      int32_t idx[3];
      int n = 0;
      while (true) {
        while (*q && is_space(*q)) q++;
        if (!*q || *q == '#') break;
        char* end = nullptr;
        errno = 0;
        const long v = std::strtol(q, &end, 10);
        if (end == q || errno == ERANGE || v == 0) {
          fail("invalid face specification");
          break;
        }
        q = end;
        while (*q && !is_space(*q)) q++;  // skip "/vt/vn"
        const long nv = (long)(m.P.size() / 3);
        const long i = v > 0 ? v - 1 : nv + v;  // negative: relative to the vertices read so far
        if (i < 0 || i >= nv) {
          fail("face index out of range");
          break;
        }
        if (n == 3) {
          fail("invalid face specification (only triangles supported)");
          break;
        }
        idx[n++] = (int32_t)i;
      }
      if (!ok) break;
      if (n != 3) {
        fail("invalid face specification (only triangles supported)");
        break;
      }
      m.E.insert(m.E.end(), idx, idx + 3);
    }
    // anything else ("vn", "vt", "vp", "#", "o", "g", "s", "usemtl", "mtllib", blank) is skipped
  }
  std::fclose(f);
  return ok;
}

thread_local std::string g_obj_err;

}  // namespace

extern "C" {

const char* ac3d_obj_last_error(void) { return g_obj_err.c_str(); }

int ac3d_read_obj(const char* path, double* Ps, int V_cap, int32_t* Es, int Ne_cap, int* V, int* Ne) {
  if (!path || !V || !Ne) return AC3D_ERR_ARG;
  ObjMesh m;
  if (!parse_obj(path, m)) {
    g_obj_err = m.err;
    return AC3D_ERR_ARG;
  }
  const size_t nv = m.P.size() / 3, ne = m.E.size() / 3;
  if (nv > 0x7fffffff || ne > 0x7fffffff) {
    g_obj_err = "mesh too large";
    return AC3D_ERR_RESOURCE;
  }
  *V = (int)nv;
  *Ne = (int)ne;
  if (!Ps && !Es) return AC3D_OK;  // size query
  if (!Ps || !Es || V_cap < (int)nv || Ne_cap < (int)ne) {
    g_obj_err = "output arrays smaller than the mesh";
    return AC3D_ERR_RESOURCE;
  }
  std::memcpy(Ps, m.P.data(), m.P.size() * sizeof(double));
  std::memcpy(Es, m.E.data(), m.E.size() * sizeof(int32_t));
  return AC3D_OK;
}

int ac3d_write_obj(const char* path, const double* Ps, int V, const int32_t* Es, int Ne) {
  if (!path || (V > 0 && !Ps) || (Ne > 0 && !Es) || V < 0 || Ne < 0) return AC3D_ERR_ARG;
  for (long i = 0; i < 3L * Ne; i++)
    if (Es[i] < 0 || Es[i] >= V) {
      g_obj_err = "face index out of range";
      return AC3D_ERR_ARG;
    }
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    g_obj_err = std::string("cannot open ") + path;
    return AC3D_ERR_ARG;
  }
  bool ok = true;
  for (long i = 0; i < V && ok; i++)
    ok = std::fprintf(f, "v %.17g %.17g %.17g\n", Ps[3 * i], Ps[3 * i + 1], Ps[3 * i + 2]) > 0;
  for (long i = 0; i < Ne && ok; i++)
    ok = std::fprintf(f, "f %d %d %d\n", Es[3 * i] + 1, Es[3 * i + 1] + 1, Es[3 * i + 2] + 1) > 0;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    g_obj_err = std::string("write failed: ") + path;
    return AC3D_ERR_INTERNAL;
  }
  return AC3D_OK;
}

}  // extern "C"
