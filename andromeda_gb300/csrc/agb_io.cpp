// Input and output formats of the reference, host code (no device work):
//
//   agb_mesh_read     the surface-mesh readers of ReadSurfaceMesh
//                     (src/lib_meshRead.f90:80-160): gmsh 2.x ASCII (ReadGMSHv2
//                     :244), gmsh 4.x ASCII (ReadGMSHv4Surface :385) and the
//                     reference's own "andromedaMesh" text format
//                     (ReadAndromedaMesh :165).  One deviation: the reference
//                     refuses a gmsh 4 file whose $Entities lists volumes
//                     (getMeshTypev4 :337 -> "invalid surface mesh file"), the
//                     mesh of its own flow-over-ellipsoid case among them; here
//                     the element blocks of dimension 2 of any gmsh 4 file are
//                     read and the other blocks skipped;
//   agb_vtu_write     the ParaView file of the results (OutputMeshParaview,
//                     src/lib_mesh.f90:218-392);
//   agb_integrals_file_write / _read
//                     the integral-matrix cache and.integrals.bin
//                     (WriteIntegralsToDisk / ReadIntegralsFile,
//                     src/lib_int.f90:136-221; the Stokes variants
//                     src/lib_Stokes.f90:2742-2876): Fortran sequential
//                     unformatted records as gfortran writes them (a 4-byte
//                     length before and after every record).
//
// Lines are read as the reference's rOneTL (src/lib_mesh.f90:1804) reads them:
// empty lines and every line holding a '#' are skipped.
#include "../../include/andromeda_gb300.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

__attribute__((visibility("hidden"))) void agb_set_free_error(const std::string& msg);

namespace {

// element types of the reference (mod_mesh.f90): 2 = 3-node triangle, 3 = 4-node quad
constexpr int AGB_TRI = 2;
constexpr int AGB_QUAD = 3;

int io_fail(int code, const std::string& msg) {
  agb_set_free_error(msg);
  return code;
}

struct LineReader {
  std::ifstream f;
  explicit LineReader(const char* path) : f(path) {}
  bool ok() const { return (bool)f; }
  // next line that is neither empty nor holds a '#'; false at the end of the file
  bool next(std::string& line) {
    while (std::getline(f, line)) {
      if (!line.empty() && line.back() == '\r') line.pop_back();
      if (line.find_first_not_of(" \t") == std::string::npos) continue;
      if (line.find('#') != std::string::npos) continue;
      return true;
    }
    return false;
  }
};

std::string trimmed(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

struct MeshData {
  std::vector<double> xyz;         // [n][3]
  std::vector<int> etype, con, bcid;  // con [e][4] 1-based while reading
  std::vector<int> wall_id;
  std::vector<std::string> wall_name;
  std::vector<char> node_set, elem_set;
};

std::string unquote(std::string s) {
  s = trimmed(s);
  if (s.size() >= 2 && (s.front() == '"' || s.front() == '\'') && s.back() == s.front()) return s.substr(1, s.size() - 2);
  return s;
}

bool set_node(MeshData& M, long j, double x, double y, double z, std::string& err) {
  const long n = (long)M.node_set.size();
  if (j < 1 || j > n) {
    err = "node tag " + std::to_string(j) + " outside 1.." + std::to_string(n);
    return false;
  }
  M.xyz[3 * (j - 1)] = x;
  M.xyz[3 * (j - 1) + 1] = y;
  M.xyz[3 * (j - 1) + 2] = z;
  M.node_set[j - 1] = 1;
  return true;
}

bool set_element(MeshData& M, long j, int type, int bcid, const long* nodes, std::string& err) {
  const long n = (long)M.elem_set.size();
  if (j < 1 || j > n) {
    err = "element tag " + std::to_string(j) + " outside 1.." + std::to_string(n);
    return false;
  }
  if (type != AGB_TRI && type != AGB_QUAD) {
    err = "element " + std::to_string(j) + ": element type " + std::to_string(type) +
          " not supported (2 = 3-node triangle, 3 = 4-node quad)";
    return false;
  }
  const int nno = type == AGB_TRI ? 3 : 4;
  M.etype[j - 1] = type;
  M.bcid[j - 1] = bcid;
  for (int k = 0; k < 4; ++k) M.con[4 * (j - 1) + k] = k < nno ? (int)nodes[k] : -1;
  M.elem_set[j - 1] = 1;
  return true;
}

void init_nodes(MeshData& M, long n) {
  M.xyz.assign(3 * (size_t)n, 0.0);
  M.node_set.assign((size_t)n, 0);
}
void init_elements(MeshData& M, long n) {
  M.etype.assign((size_t)n, 0);
  M.bcid.assign((size_t)n, 0);
  M.con.assign(4 * (size_t)n, -1);
  M.elem_set.assign((size_t)n, 0);
}

// ReadGMSHv2 (lib_meshRead.f90:244-330)
bool read_gmsh2(LineReader& R, MeshData& M, std::string& err) {
  std::string line;
  while (R.next(line)) {
    const std::string t = trimmed(line);
    if (t == "$Nodes") {
      if (!R.next(line)) break;
      const long n = std::stol(line);
      init_nodes(M, n);
      for (long i = 0; i < n; ++i) {
        if (!R.next(line)) { err = "end of file in $Nodes"; return false; }
        std::istringstream s(line);
        long j;
        double x, y, z;
        if (!(s >> j >> x >> y >> z)) { err = "bad node line: " + line; return false; }
        if (!set_node(M, j, x, y, z, err)) return false;
      }
    } else if (t == "$Elements") {
      if (!R.next(line)) break;
      const long n = std::stol(line);
      init_elements(M, n);
      for (long i = 0; i < n; ++i) {
        if (!R.next(line)) { err = "end of file in $Elements"; return false; }
        std::istringstream s(line);
        long j;
        int type, ntags;
        if (!(s >> j >> type >> ntags)) { err = "bad element line: " + line; return false; }
        std::vector<long> tags((size_t)std::max(ntags, 0));
        for (auto& v : tags)
          if (!(s >> v)) { err = "bad element line: " + line; return false; }
        const int bc = ntags > 0 ? (int)tags[0] : 0;
        long nodes[4] = {0, 0, 0, 0};
        const int nno = type == AGB_QUAD ? 4 : 3;
        for (int k = 0; k < nno && (type == AGB_TRI || type == AGB_QUAD); ++k)
          if (!(s >> nodes[k])) { err = "bad element line: " + line; return false; }
        if (!set_element(M, j, type, bc, nodes, err)) return false;
      }
    } else if (t == "$PhysicalNames") {
      if (!R.next(line)) break;
      const long n = std::stol(line);
      for (long i = 0; i < n; ++i) {
        if (!R.next(line)) { err = "end of file in $PhysicalNames"; return false; }
        std::istringstream s(line);
        int dim, id;
        if (!(s >> dim >> id)) { err = "bad physical name line: " + line; return false; }
        std::string rest;
        std::getline(s, rest);
        M.wall_id.push_back(id);
        M.wall_name.push_back(unquote(rest));
      }
    }
  }
  return true;
}

// ReadGMSHv4Surface (lib_meshRead.f90:385-560)
bool read_gmsh4_surface(LineReader& R, MeshData& M, std::string& err) {
  std::string line;
  std::vector<std::pair<long, int>> ent2phy;  // surface tag -> |physical tag|
  while (R.next(line)) {
    const std::string t = trimmed(line);
    if (t == "$Entities") {
      if (!R.next(line)) break;
      long np = 0, nc = 0, ns = 0, nv = 0;
      std::istringstream(line) >> np >> nc >> ns >> nv;
      for (long i = 0; i < np + nc; ++i)
        if (!R.next(line)) { err = "end of file in $Entities"; return false; }
      for (long i = 0; i < ns; ++i) {
        if (!R.next(line)) { err = "end of file in $Entities"; return false; }
        std::istringstream s(line);
        long tag, nphys = 0, phys = 0;
        double bb[6];
        s >> tag;
        for (double& v : bb) s >> v;
        s >> nphys >> phys;  // the first physical tag (the reference reads the 9th value either way)
        ent2phy.push_back({tag, (int)std::labs(phys)});
      }
      for (long i = 0; i < nv; ++i)
        if (!R.next(line)) { err = "end of file in $Entities"; return false; }
    } else if (t == "$Nodes") {
      if (!R.next(line)) break;
      long nblocks = 0, n = 0, mn = 0, mx = 0;
      std::istringstream(line) >> nblocks >> n >> mn >> mx;
      init_nodes(M, n);
      for (long b = 0; b < nblocks; ++b) {
        if (!R.next(line)) { err = "end of file in $Nodes"; return false; }
        long dim, etag, param, nin = 0;
        std::istringstream(line) >> dim >> etag >> param >> nin;
        std::vector<long> tags((size_t)nin);
        for (auto& v : tags) {
          if (!R.next(line)) { err = "end of file in $Nodes"; return false; }
          v = std::stol(line);
        }
        for (long k = 0; k < nin; ++k) {
          if (!R.next(line)) { err = "end of file in $Nodes"; return false; }
          double x, y, z;
          std::istringstream s(line);
          if (!(s >> x >> y >> z)) { err = "bad node line: " + line; return false; }
          if (!set_node(M, tags[(size_t)k], x, y, z, err)) return false;
        }
      }
    } else if (t == "$Elements") {
      if (!R.next(line)) break;
      long nblocks = 0, n = 0, mn = 0, mx = 0;
      std::istringstream(line) >> nblocks >> n >> mn >> mx;
      init_elements(M, std::max(n, mx));  // by tag; compacted below when blocks were skipped
      int phys = 0;  // kept from the previous block when the entity is no surface, as the reference does
      for (long b = 0; b < nblocks; ++b) {
        if (!R.next(line)) { err = "end of file in $Elements"; return false; }
        long dim, etag, nin = 0;
        int type;
        std::istringstream(line) >> dim >> etag >> type >> nin;
        if (dim != 2) {  // points, lines or volume cells: not surface elements
          for (long k = 0; k < nin; ++k)
            if (!R.next(line)) { err = "end of file in $Elements"; return false; }
          continue;
        }
        for (const auto& p : ent2phy)
          if (p.first == etag) phys = p.second;
        for (long k = 0; k < nin; ++k) {
          if (!R.next(line)) { err = "end of file in $Elements"; return false; }
          std::istringstream s(line);
          long j, nodes[4] = {0, 0, 0, 0};
          s >> j;
          const int nno = type == AGB_QUAD ? 4 : 3;
          for (int q = 0; q < nno && (type == AGB_TRI || type == AGB_QUAD); ++q)
            if (!(s >> nodes[q])) { err = "bad element line: " + line; return false; }
          if (!set_element(M, j, type, phys, nodes, err)) return false;
        }
      }
    } else if (t == "$PhysicalNames") {
      if (!R.next(line)) break;
      const long n = std::stol(line);
      for (long i = 0; i < n; ++i) {
        if (!R.next(line)) { err = "end of file in $PhysicalNames"; return false; }
        std::istringstream s(line);
        int dim, id;
        if (!(s >> dim >> id)) { err = "bad physical name line: " + line; return false; }
        std::string rest;
        std::getline(s, rest);
        M.wall_id.push_back(id);
        M.wall_name.push_back(unquote(rest));
      }
    }
  }
  // the surface elements in tag order (all tags when no block was skipped)
  size_t k = 0;
  for (size_t e = 0; e < M.elem_set.size(); ++e) {
    if (!M.elem_set[e]) continue;
    M.etype[k] = M.etype[e];
    M.bcid[k] = M.bcid[e];
    for (int q = 0; q < 4; ++q) M.con[4 * k + q] = M.con[4 * e + q];
    M.elem_set[k] = 1;
    ++k;
  }
  M.etype.resize(k);
  M.bcid.resize(k);
  M.con.resize(4 * k);
  M.elem_set.resize(k);
  return true;
}

// ReadAndromedaMesh (lib_meshRead.f90:165-240): header, version, walls, nodes, elements
bool read_andromeda(LineReader& R, MeshData& M, std::string& err) {
  std::string line;
  if (!R.next(line) || !R.next(line)) { err = "andromedaMesh: missing header"; return false; }
  if (!R.next(line)) { err = "andromedaMesh: missing walls"; return false; }
  const long nw = std::stol(line);
  for (long i = 0; i < nw; ++i) {
    if (!R.next(line)) { err = "andromedaMesh: end of file in the walls"; return false; }
    std::istringstream s(line);
    int id;
    s >> id;
    std::string rest;
    std::getline(s, rest);
    M.wall_id.push_back(id);
    M.wall_name.push_back(unquote(rest));
  }
  if (!R.next(line)) { err = "andromedaMesh: missing nodes"; return false; }
  const long nn = std::stol(line);
  init_nodes(M, nn);
  for (long i = 0; i < nn; ++i) {
    if (!R.next(line)) { err = "andromedaMesh: end of file in the nodes"; return false; }
    std::istringstream s(line);
    long j;
    double x, y, z;
    if (!(s >> j >> x >> y >> z)) { err = "bad node line: " + line; return false; }
    if (!set_node(M, j, x, y, z, err)) return false;
  }
  if (!R.next(line)) { err = "andromedaMesh: missing elements"; return false; }
  const long ne = std::stol(line);
  init_elements(M, ne);
  for (long i = 0; i < ne; ++i) {
    if (!R.next(line)) { err = "andromedaMesh: end of file in the elements"; return false; }
    std::istringstream s(line);
    long j, nodes[4] = {0, 0, 0, 0};
    int bc, nno;
    if (!(s >> j >> bc >> nno)) { err = "bad element line: " + line; return false; }
    if (nno != 3 && nno != 4) { err = "andromedaMesh: element " + std::to_string(j) + " has " + std::to_string(nno) + " nodes"; return false; }
    for (int k = 0; k < nno; ++k)
      if (!(s >> nodes[k])) { err = "bad element line: " + line; return false; }
    if (!set_element(M, j, nno == 3 ? AGB_TRI : AGB_QUAD, bc, nodes, err)) return false;
  }
  return true;
}

}  // namespace

extern "C" int agb_mesh_read(const char* path, int* sizes, double* xyz, int* etype, int* con, int* bcid,
                             int* wall_ids, char* wall_names, int name_len) {
  agb_set_free_error("");
  if (!path || !sizes) return io_fail(AGB_ERR_ARG, "agb_mesh_read: path and sizes are required");
  LineReader R(path);
  if (!R.ok()) return io_fail(AGB_ERR_ARG, std::string("agb_mesh_read: cannot open ") + path);
  std::string first, err;
  MeshData M;
  bool ok = false;
  if (!R.next(first)) return io_fail(AGB_ERR_ARG, "agb_mesh_read: empty file");
  const std::string head = trimmed(first);
  try {
    if (head == "andromedaMesh") {
      LineReader R2(path);
      ok = read_andromeda(R2, M, err);
    } else if (head == "$MeshFormat") {
      std::string vline;
      if (!R.next(vline)) return io_fail(AGB_ERR_ARG, "agb_mesh_read: no version after $MeshFormat");
      double version = 0.0;
      int file_type = 0;
      std::istringstream(vline) >> version >> file_type;
      if (file_type != 0) return io_fail(AGB_ERR_UNSUPPORTED, "agb_mesh_read: binary gmsh files are not read (ASCII only)");
      LineReader R2(path);
      if (version < 4.0) ok = read_gmsh2(R2, M, err);
      else ok = read_gmsh4_surface(R2, M, err);
    } else {
      return io_fail(AGB_ERR_ARG, "agb_mesh_read: invalid surface mesh file (neither $MeshFormat nor andromedaMesh)");
    }
  } catch (const std::exception& e) {
    return io_fail(AGB_ERR_ARG, std::string("agb_mesh_read: unreadable number: ") + e.what());
  }
  if (!ok) return io_fail(AGB_ERR_ARG, "agb_mesh_read: " + err);
  for (size_t i = 0; i < M.node_set.size(); ++i)
    if (!M.node_set[i]) return io_fail(AGB_ERR_ARG, "agb_mesh_read: node " + std::to_string(i + 1) + " is missing");
  for (size_t e = 0; e < M.elem_set.size(); ++e)
    if (!M.elem_set[e]) return io_fail(AGB_ERR_ARG, "agb_mesh_read: element " + std::to_string(e + 1) + " is missing");
  const int nn = (int)M.node_set.size(), ne = (int)M.elem_set.size(), nw = (int)M.wall_id.size();
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < (M.etype[e] == AGB_TRI ? 3 : 4); ++k) {
      const int v = M.con[4 * (size_t)e + k];
      if (v < 1 || v > nn)
        return io_fail(AGB_ERR_ARG, "agb_mesh_read: element " + std::to_string(e + 1) + " names node " +
                                        std::to_string(v) + " outside 1.." + std::to_string(nn));
    }
  sizes[0] = nn;
  sizes[1] = ne;
  sizes[2] = nw;
  if (!xyz) return AGB_OK;  // size query
  if (!etype || !con || !bcid) return io_fail(AGB_ERR_ARG, "agb_mesh_read: output arrays missing");
  std::memcpy(xyz, M.xyz.data(), M.xyz.size() * sizeof(double));
  for (int e = 0; e < ne; ++e) {
    etype[e] = M.etype[e];
    bcid[e] = M.bcid[e];
    for (int k = 0; k < 4; ++k) {
      const int v = M.con[4 * (size_t)e + k];
      con[4 * (size_t)e + k] = v > 0 ? v - 1 : -1;  // 0-based, -1 = no fourth node
    }
  }
  if (wall_ids)
    for (int i = 0; i < nw; ++i) wall_ids[i] = M.wall_id[i];
  if (wall_names && name_len > 0)
    for (int i = 0; i < nw; ++i) {
      char* d = wall_names + (size_t)i * name_len;
      std::memset(d, 0, (size_t)name_len);
      std::strncpy(d, M.wall_name[i].c_str(), (size_t)name_len - 1);
    }
  return AGB_OK;
}

namespace {
// a value as the ParaView file carries it (Float32 data arrays, 9 significant digits)
void put(FILE* f, double v) { std::fprintf(f, "%.9g\n", v); }
}  // namespace

// OutputMeshParaview (lib_mesh.f90:218-392)
extern "C" int agb_vtu_write(const char* path, int kind, int nnodes, const double* xyz, int nelem, const int* etype,
                             const int* con, const int* bcid, const double* normal, int neq, const char* const* names,
                             const double* u, const double* q, const double* p) {
  agb_set_free_error("");
  if (!path || nnodes < 1 || nelem < 1 || !xyz || !etype || !con || !bcid || !normal || neq < 1 || !names || !u || !q)
    return io_fail(AGB_ERR_ARG, "agb_vtu_write: missing arguments");
  if (kind != AGB_LAPLACE && kind != AGB_STOKES) return io_fail(AGB_ERR_ARG, "agb_vtu_write: kind must be Laplace or Stokes");
  if (kind == AGB_STOKES && (neq != 3 || !p)) return io_fail(AGB_ERR_ARG, "agb_vtu_write: Stokes needs neq = 3 and the pressure");
  for (int e = 0; e < nelem; ++e)
    if (etype[e] != AGB_TRI && etype[e] != AGB_QUAD) return io_fail(AGB_ERR_ARG, "agb_vtu_write: element type not supported");
  FILE* f = std::fopen(path, "w");
  if (!f) return io_fail(AGB_ERR_ARG, std::string("agb_vtu_write: cannot create ") + path);
  std::fprintf(f, "<?xml version=\"1.0\"?>\n");
  std::fprintf(f, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\" "
                  "compressor=\"vtkZLibDataCompressor\">\n<UnstructuredGrid>\n");
  std::fprintf(f, "<Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n", nnodes, nelem);
  std::string ulist, qlist;
  for (int j = 0; j < neq; ++j) {
    ulist += std::string(",u") + names[j];
    qlist += std::string(",q") + names[j];
  }
  if (kind == AGB_STOKES) std::fprintf(f, "<PointData Vectors=\"u\" Scalars=\"node%s\">\n", ulist.c_str());
  else std::fprintf(f, "<PointData Scalars=\"node%s\">\n", ulist.c_str());
  if (kind == AGB_STOKES) {
    std::fprintf(f, "<DataArray type=\"Float32\" Name=\"u\" NumberOfComponents=\"3\" format=\"ascii\">\n");
    for (int i = 0; i < nnodes; ++i)
      std::fprintf(f, "%.9g %.9g %.9g\n", u[i], u[(size_t)nnodes + i], u[2 * (size_t)nnodes + i]);
    std::fprintf(f, "</DataArray>\n");
  }
  std::fprintf(f, "<DataArray type=\"Float32\" Name=\"node\" format=\"ascii\">\n");
  for (int i = 0; i < nnodes; ++i) std::fprintf(f, "%d\n", i + 1);
  std::fprintf(f, "</DataArray>\n");
  for (int j = 0; j < neq; ++j) {
    std::fprintf(f, "<DataArray type=\"Float32\" Name=\"u%s\" format=\"ascii\">\n", names[j]);
    for (int i = 0; i < nnodes; ++i) put(f, u[(size_t)j * nnodes + i]);
    std::fprintf(f, "</DataArray>\n");
  }
  std::fprintf(f, "</PointData>\n");
  if (kind == AGB_STOKES) std::fprintf(f, "<CellData Vectors=\"normale\" Scalars=\"pressure,elemBCid%s\">\n", qlist.c_str());
  else std::fprintf(f, "<CellData Vectors=\"normale\" Scalars=\"elemBCid%s\">\n", qlist.c_str());
  std::fprintf(f, "<DataArray type=\"Float32\" Name=\"normale\" NumberOfComponents=\"3\" format=\"ascii\">\n");
  for (int e = 0; e < nelem; ++e)
    std::fprintf(f, "%.9g %.9g %.9g\n", normal[3 * (size_t)e], normal[3 * (size_t)e + 1], normal[3 * (size_t)e + 2]);
  std::fprintf(f, "</DataArray>\n");
  if (kind == AGB_STOKES) {
    std::fprintf(f, "<DataArray type=\"Float32\" Name=\"pressure\" format=\"ascii\">\n");
    for (int e = 0; e < nelem; ++e) put(f, p[e]);
    std::fprintf(f, "</DataArray>\n");
  }
  std::fprintf(f, "<DataArray type=\"Float32\" Name=\"elemBCid\" format=\"ascii\">\n");
  for (int e = 0; e < nelem; ++e) std::fprintf(f, "%d\n", bcid[e]);
  std::fprintf(f, "</DataArray>\n");
  for (int j = 0; j < neq; ++j) {
    std::fprintf(f, "<DataArray type=\"Float32\" Name=\"q%s\" format=\"ascii\">\n", names[j]);
    for (int e = 0; e < nelem; ++e) put(f, q[(size_t)j * nelem + e]);
    std::fprintf(f, "</DataArray>\n");
  }
  std::fprintf(f, "</CellData>\n<Points>\n<DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n");
  for (int i = 0; i < nnodes; ++i)
    std::fprintf(f, "%.9g %.9g %.9g\n", xyz[3 * (size_t)i], xyz[3 * (size_t)i + 1], xyz[3 * (size_t)i + 2]);
  std::fprintf(f, "</DataArray>\n</Points>\n<Cells>\n<DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n");
  for (int e = 0; e < nelem; ++e) {
    const int nno = etype[e] == AGB_TRI ? 3 : 4;
    for (int k = 0; k < nno; ++k) std::fprintf(f, k ? " %d" : "%d", con[4 * (size_t)e + k]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "</DataArray>\n<DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n");
  long off = 0;
  for (int e = 0; e < nelem; ++e) {
    off += etype[e] == AGB_TRI ? 3 : 4;
    std::fprintf(f, "%ld\n", off);
  }
  std::fprintf(f, "</DataArray>\n<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n");
  for (int e = 0; e < nelem; ++e) std::fprintf(f, "%d\n", etype[e] == AGB_TRI ? 5 : 9);  // VTK triangle / quad
  std::fprintf(f, "</DataArray>\n</Cells>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n");
  const bool bad = std::ferror(f) != 0;
  if (std::fclose(f) != 0 || bad) return io_fail(AGB_ERR_ARG, std::string("agb_vtu_write: write error on ") + path);
  return AGB_OK;
}

// ---------------------------------------------------------------------------
// and.integrals.bin: Fortran sequential unformatted records (gfortran: an int32
// byte count before and after each record).  Laplace (WriteIntegralsToDisk,
// lib_int.f90:185-221): (nsp, nnodes, nqnodes) int32, (FspCerr, QspCerr)
// real(8), then Hmat and Gmat column by column, each column in records of at
// most 8192 values (WrSMat / wrvec, lib_util.f90:201-290; a column whose length
// is a multiple of 8192 ends with an empty record, as wrvec writes it).  Stokes
// (WriteIntegralsToDiskStokes, lib_Stokes.f90:2742-2800): first the int32
// parStokes = 1407 (mod_par.f90:109), then the same records with the matrices
// Txx,Tyy,Tzz,Txy,Txz,Tyz, Gxx,Gyy,Gzz,Gxy,Gxz,Gyz, prTx,prTy,prTz,
// prGx,prGy,prGz.  The matrices here are those of agb_integral_matrices
// (components xx,xy,xz,yy,yz,zz,prx,pry,prz, each column-major nsp x ncol).
// ---------------------------------------------------------------------------
namespace {
constexpr int kParStokes = 1407;
constexpr int kChunk = 8192;
// component order of the Stokes file, as indices into the T (or G) components
constexpr int kFileOrder[6] = {0, 3, 5, 1, 2, 4};

bool put_record(FILE* f, const void* data, int32_t bytes) {
  return std::fwrite(&bytes, 4, 1, f) == 1 && (bytes == 0 || std::fwrite(data, (size_t)bytes, 1, f) == 1) &&
         std::fwrite(&bytes, 4, 1, f) == 1;
}
bool put_matrix(FILE* f, const double* m, int nrow, int ncol) {
  for (int j = 0; j < ncol; ++j) {
    const double* col = m + (size_t)j * nrow;
    const int nblock = nrow / kChunk;
    for (int b = 0; b < nblock; ++b)
      if (!put_record(f, col + (size_t)b * kChunk, kChunk * 8)) return false;
    const int rest = nrow - nblock * kChunk;
    if (!put_record(f, col + (size_t)nblock * kChunk, rest * 8)) return false;
  }
  return true;
}
// one record into dst (exactly `bytes` long), false on a length mismatch or a short file
bool get_record(FILE* f, void* dst, int32_t bytes) {
  int32_t a = -1, b = -1;
  if (std::fread(&a, 4, 1, f) != 1 || a != bytes) return false;
  if (bytes > 0 && std::fread(dst, (size_t)bytes, 1, f) != 1) return false;
  return std::fread(&b, 4, 1, f) == 1 && b == bytes;
}
bool get_matrix(FILE* f, double* m, int nrow, int ncol) {
  for (int j = 0; j < ncol; ++j) {
    double* col = m + (size_t)j * nrow;
    const int nblock = nrow / kChunk;
    for (int b = 0; b < nblock; ++b)
      if (!get_record(f, col + (size_t)b * kChunk, kChunk * 8)) return false;
    const int rest = nrow - nblock * kChunk;
    if (!get_record(f, col + (size_t)nblock * kChunk, rest * 8)) return false;
  }
  return true;
}
}  // namespace

extern "C" int agb_integrals_file_write(const char* path, int kind, int nsp, int nnodes, int nqnodes,
                                        const double* errs, const double* T, const double* G) {
  agb_set_free_error("");
  if (!path || nsp < 1 || nnodes < 1 || nqnodes < 1 || !errs || !T || !G)
    return io_fail(AGB_ERR_ARG, "agb_integrals_file_write: missing arguments");
  if (kind != AGB_LAPLACE && kind != AGB_STOKES) return io_fail(AGB_ERR_ARG, "agb_integrals_file_write: bad kind");
  FILE* f = std::fopen(path, "wb");
  if (!f) return io_fail(AGB_ERR_ARG, std::string("agb_integrals_file_write: cannot create ") + path);
  bool ok = true;
  if (kind == AGB_STOKES) ok = put_record(f, &kParStokes, 4);
  const int32_t sz[3] = {nsp, nnodes, nqnodes};
  ok = ok && put_record(f, sz, 12) && put_record(f, errs, 16);
  const size_t mt = (size_t)nsp * nnodes, mg = (size_t)nsp * nqnodes;
  if (kind == AGB_LAPLACE) {
    ok = ok && put_matrix(f, T, nsp, nnodes) && put_matrix(f, G, nsp, nqnodes);
  } else {
    for (int k = 0; k < 6 && ok; ++k) ok = put_matrix(f, T + kFileOrder[k] * mt, nsp, nnodes);
    for (int k = 0; k < 6 && ok; ++k) ok = put_matrix(f, G + kFileOrder[k] * mg, nsp, nqnodes);
    for (int k = 6; k < 9 && ok; ++k) ok = put_matrix(f, T + k * mt, nsp, nnodes);
    for (int k = 6; k < 9 && ok; ++k) ok = put_matrix(f, G + k * mg, nsp, nqnodes);
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return io_fail(AGB_ERR_ARG, std::string("agb_integrals_file_write: write error on ") + path);
  return AGB_OK;
}

extern "C" int agb_integrals_file_read(const char* path, int kind, int* sizes, double* errs, double* T, double* G) {
  agb_set_free_error("");
  if (!path || !sizes) return io_fail(AGB_ERR_ARG, "agb_integrals_file_read: missing arguments");
  if (kind != AGB_LAPLACE && kind != AGB_STOKES) return io_fail(AGB_ERR_ARG, "agb_integrals_file_read: bad kind");
  FILE* f = std::fopen(path, "rb");
  if (!f) return io_fail(AGB_ERR_ARG, std::string("agb_integrals_file_read: cannot open ") + path);
  int32_t tag = 0, sz[3] = {0, 0, 0};
  double e[2] = {0.0, 0.0};
  bool ok = true;
  if (kind == AGB_STOKES) ok = get_record(f, &tag, 4) && tag == kParStokes;
  ok = ok && get_record(f, sz, 12) && sz[0] > 0 && sz[1] > 0 && sz[2] > 0 && get_record(f, e, 16);
  if (ok && T && G) {
    // the caller's sizes must match the file's (ReadIntegralsFile, lib_int.f90:152-157)
    if (sz[0] != sizes[0] || sz[1] != sizes[1] || sz[2] != sizes[2]) {
      std::fclose(f);
      return io_fail(AGB_ERR_ARG, "agb_integrals_file_read: the file's sizes do not match");
    }
    const int nsp = sz[0], nn = sz[1], nq = sz[2];
    const size_t mt = (size_t)nsp * nn, mg = (size_t)nsp * nq;
    if (kind == AGB_LAPLACE) {
      ok = get_matrix(f, T, nsp, nn) && get_matrix(f, G, nsp, nq);
    } else {
      for (int k = 0; k < 6 && ok; ++k) ok = get_matrix(f, T + kFileOrder[k] * mt, nsp, nn);
      for (int k = 0; k < 6 && ok; ++k) ok = get_matrix(f, G + kFileOrder[k] * mg, nsp, nq);
      for (int k = 6; k < 9 && ok; ++k) ok = get_matrix(f, T + k * mt, nsp, nn);
      for (int k = 6; k < 9 && ok; ++k) ok = get_matrix(f, G + k * mg, nsp, nq);
    }
  }
  std::fclose(f);
  if (!ok) return io_fail(AGB_ERR_ARG, std::string("agb_integrals_file_read: not an integrals file of this kind: ") + path);
  for (int i = 0; i < 3; ++i) sizes[i] = sz[i];
  if (errs) {
    errs[0] = e[0];
    errs[1] = e[1];
  }
  return AGB_OK;
}
