// ggem_io.cpp -- particle files in the reference's formats (include/ggem_io.h).
//
// The layouts are the reference's (they are the interface to COPSS input
// decks and to its post-processing): the LAMMPS-style data file of
// PolymerChain::read_particles_data, the polydata VTK of
// write_polymer_trajectory / read_data_vtk, the bead CSV of
// write_bead_trajectory, and PETSc's binary vector file for restarts.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

#include "ggem_gb300.h"
#include "ggem_io.h"

namespace {

template <typename T>
T *dup(const std::vector<T> &v) {
  if (v.empty()) return nullptr;
  T *p = static_cast<T *>(std::malloc(sizeof(T) * v.size()));
  if (p) std::memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}

std::string trim(const std::string &s) {
  const size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  const size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

// the next line whose trimmed text equals `key`
bool seek_section(std::istream &in, const char *key) {
  std::string line;
  while (std::getline(in, line))
    if (trim(line) == key) return true;
  return false;
}

// "value word [word]" header line: value and the words
bool header_count(std::istream &in, int64_t *v, const char *w1, const char *w2) {
  std::string line;
  while (std::getline(in, line)) {
    if (trim(line).empty()) continue;
    std::istringstream ss(line);
    std::string a, b;
    if (!(ss >> *v >> a)) return false;
    if (a != w1) return false;
    if (w2) {
      if (!(ss >> b) || b != w2) return false;
    }
    return true;
  }
  return false;
}

void put_be32(std::ostream &o, uint32_t v) {
  unsigned char b[4] = {(unsigned char)(v >> 24), (unsigned char)(v >> 16),
                        (unsigned char)(v >> 8), (unsigned char)v};
  o.write(reinterpret_cast<const char *>(b), 4);
}
bool get_be32(std::istream &i, uint32_t *v) {
  unsigned char b[4];
  if (!i.read(reinterpret_cast<char *>(b), 4)) return false;
  *v = ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | b[3];
  return true;
}

constexpr uint32_t kPetscVecClassId = 1211214;

}  // namespace

extern "C" void ggem_free_polymer_data(ggem_polymer_data *d) {
  if (!d) return;
  std::free(d->xyz);
  std::free(d->chain_id);
  std::free(d->bead_type);
  std::free(d->rot);
  std::free(d->const_force);
  std::free(d->charge);
  std::free(d->mass);
  std::free(d->bonds);
  std::free(d->bond_type);
  std::memset(d, 0, sizeof(*d));
}

extern "C" int ggem_read_polymer_data(const char *path, ggem_polymer_data *out) {
  if (!path || !out) return GGEM_ERR_BAD_ARG;
  std::memset(out, 0, sizeof(*out));
  std::ifstream in(path);
  if (!in.good()) return GGEM_ERR_BAD_ARG;
  std::string line;
  std::getline(in, line);  // header line
  int64_t nb = 0, nbond = 0, nt = 0, nbt = 0;
  if (!header_count(in, &nb, "atoms", nullptr) || !header_count(in, &nbond, "bonds", nullptr) ||
      !header_count(in, &nt, "atom", "types") || !header_count(in, &nbt, "bond", "types") ||
      nb < 0 || nbond < 0 || nt < 1 || nbt < 0)
    return GGEM_ERR_BAD_ARG;
  // optional box lines ("lo hi xlo xhi"), then Masses
  while (std::getline(in, line)) {
    const std::string t = trim(line);
    if (t == "Masses") break;
    std::istringstream ss(t);
    double lo, hi;
    std::string a, b;
    if (ss >> lo >> hi >> a >> b) {
      const int d = a == "xlo" ? 0 : a == "ylo" ? 1 : a == "zlo" ? 2 : -1;
      if (d >= 0) {
        out->box_lo[d] = lo;
        out->box_hi[d] = hi;
        out->has_box = 1;
      }
    }
  }
  if (!in) return GGEM_ERR_BAD_ARG;
  std::vector<double> mass((size_t)nt);
  for (int64_t k = 0; k < nt; ++k) {
    int64_t id;
    if (!(in >> id >> mass[k])) return GGEM_ERR_BAD_ARG;
  }
  if (!seek_section(in, "Atoms")) return GGEM_ERR_BAD_ARG;
  std::vector<double> xyz(3 * nb), rot(3 * nb), cf(3 * nb), q(nb);
  std::vector<int32_t> chain(nb), type(nb);
  int max_chain = 0;
  for (int64_t i = 0; i < nb; ++i) {
    int64_t id, c, t;
    if (!(in >> id >> c >> t >> xyz[3 * i] >> xyz[3 * i + 1] >> xyz[3 * i + 2] >> rot[3 * i] >>
          rot[3 * i + 1] >> rot[3 * i + 2] >> cf[3 * i] >> cf[3 * i + 1] >> cf[3 * i + 2] >> q[i]))
      return GGEM_ERR_BAD_ARG;
    if (id != i + 1) return GGEM_ERR_BAD_ARG;  // beads listed in id order
    chain[i] = (int32_t)(c - 1);
    type[i] = (int32_t)(t - 1);
    if (c > max_chain) max_chain = (int)c;
  }
  std::vector<int64_t> bonds(2 * nbond);
  std::vector<int32_t> btype(nbond);
  if (nbond > 0) {
    if (!seek_section(in, "Bonds")) return GGEM_ERR_BAD_ARG;
    for (int64_t k = 0; k < nbond; ++k) {
      int64_t id, t, a, b;
      if (!(in >> id >> t >> a >> b) || a < 1 || a > nb || b < 1 || b > nb)
        return GGEM_ERR_BAD_ARG;
      btype[k] = (int32_t)(t - 1);
      bonds[2 * k] = a - 1;
      bonds[2 * k + 1] = b - 1;
    }
  }
  out->n_beads = nb;
  out->n_bonds = nbond;
  out->n_bead_types = (int)nt;
  out->n_bond_types = (int)nbt;
  out->n_chains = max_chain;
  out->xyz = dup(xyz);
  out->rot = dup(rot);
  out->const_force = dup(cf);
  out->charge = dup(q);
  out->chain_id = dup(chain);
  out->bead_type = dup(type);
  out->mass = dup(mass);
  out->bonds = dup(bonds);
  out->bond_type = dup(btype);
  return GGEM_OK;
}

extern "C" int ggem_read_polymer_vtk(const char *path, ggem_polymer_data *out) {
  if (!path || !out) return GGEM_ERR_BAD_ARG;
  std::memset(out, 0, sizeof(*out));
  std::ifstream in(path);
  if (!in.good()) return GGEM_ERR_BAD_ARG;
  std::string line, word, kind;
  for (int k = 0; k < 4; ++k) std::getline(in, line);  // header, title, ASCII, DATASET
  int64_t nb = 0;
  if (!(in >> word >> nb >> kind) || word != "POINTS" || nb < 0) return GGEM_ERR_BAD_ARG;
  std::vector<double> xyz(3 * nb);
  for (int64_t i = 0; i < 3 * nb; ++i)
    if (!(in >> xyz[i])) return GGEM_ERR_BAD_ARG;
  int64_t nbond = 0, size = 0;
  if (!(in >> word >> nbond >> size) || word != "LINES" || nbond < 0) return GGEM_ERR_BAD_ARG;
  std::vector<int64_t> bonds(2 * nbond);
  for (int64_t k = 0; k < nbond; ++k) {
    int64_t two;
    if (!(in >> two >> bonds[2 * k] >> bonds[2 * k + 1]) || two != 2) return GGEM_ERR_BAD_ARG;
  }
  std::vector<int32_t> chain(nb, 0);
  int max_chain = -1;
  if (seek_section(in, "LOOKUP_TABLE default")) {
    for (int64_t i = 0; i < nb; ++i) {
      int64_t c;
      if (!(in >> c)) return GGEM_ERR_BAD_ARG;
      chain[i] = (int32_t)c;
      if (c > max_chain) max_chain = (int)c;
    }
  }
  out->n_beads = nb;
  out->n_bonds = nbond;
  out->n_bead_types = 1;
  out->n_bond_types = 1;
  out->n_chains = max_chain + 1;
  out->xyz = dup(xyz);
  out->chain_id = dup(chain);
  out->bead_type = dup(std::vector<int32_t>(nb, 0));
  out->bonds = dup(bonds);
  out->bond_type = dup(std::vector<int32_t>(nbond, 0));
  return GGEM_OK;
}

extern "C" int ggem_write_polymer_vtk(const char *path, int64_t n, const double *xyz, int64_t m,
                                      const int64_t *bonds, const int32_t *chain_id,
                                      int precision) {
  if (!path || n < 0 || m < 0 || (n && !xyz) || (m && !bonds) || precision < 0)
    return GGEM_ERR_BAD_ARG;
  std::ofstream o(path);
  if (!o.good()) return GGEM_ERR_BAD_ARG;
  o.precision(precision);
  o.setf(std::ios::fixed);
  o << "# vtk DataFile Version 4.0\n"
    << "Polymer chain\n"
    << "ASCII\n"
    << "DATASET POLYDATA\n";
  o << "POINTS " << n << " float\n";
  for (int64_t i = 0; i < n; ++i) {
    for (int d = 0; d < 3; ++d) o << xyz[3 * i + d] << " ";
    o << "\n";
  }
  o << "\n";
  o << "LINES " << m << " " << m * 3 << "\n";
  for (int64_t k = 0; k < m; ++k) o << 2 << " " << bonds[2 * k] << " " << bonds[2 * k + 1] << "\n";
  o << "POINT_DATA " << n << "\n";
  o << "SCALARS bead_type int\n";
  o << "LOOKUP_TABLE default \n";
  for (int64_t i = 0; i < n; ++i) o << (chain_id ? chain_id[i] : 0) << " \n";
  return o.good() ? GGEM_OK : GGEM_ERR_BAD_ARG;
}

extern "C" int ggem_write_bead_csv(const char *path, int64_t n, const double *xyz,
                                   const double *vel, const double *force, int precision) {
  if (!path || n < 0 || (n && !xyz) || precision < 0) return GGEM_ERR_BAD_ARG;
  std::ofstream o(path);
  if (!o.good()) return GGEM_ERR_BAD_ARG;
  o << "scalar x_coord y_coord z_coord x_vel y_vel z_vel x_force y_force z_force\n";
  o.precision(precision);
  for (int64_t i = 0; i < n; ++i) {
    o << i << " ";
    for (int d = 0; d < 3; ++d) o << xyz[3 * i + d] << " ";
    for (int d = 0; d < 3; ++d) o << (vel ? vel[3 * i + d] : 0.0) << " ";
    for (int d = 0; d < 3; ++d) o << (force ? force[3 * i + d] : 0.0) << " ";
    o << "\n";
  }
  o << "\n";
  return o.good() ? GGEM_OK : GGEM_ERR_BAD_ARG;
}

extern "C" int ggem_write_petsc_vec(const char *path, int64_t n, const double *v) {
  if (!path || n < 0 || n > INT32_MAX || (n && !v)) return GGEM_ERR_BAD_ARG;
  std::ofstream o(path, std::ios::binary);
  if (!o.good()) return GGEM_ERR_BAD_ARG;
  put_be32(o, kPetscVecClassId);
  put_be32(o, (uint32_t)n);
  for (int64_t i = 0; i < n; ++i) {
    uint64_t b;
    std::memcpy(&b, v + i, 8);
    unsigned char c[8];
    for (int k = 0; k < 8; ++k) c[k] = (unsigned char)(b >> (56 - 8 * k));
    o.write(reinterpret_cast<const char *>(c), 8);
  }
  return o.good() ? GGEM_OK : GGEM_ERR_BAD_ARG;
}

extern "C" int ggem_read_petsc_vec(const char *path, int64_t n_expected, double *v,
                                   int64_t *n_read) {
  if (!path) return GGEM_ERR_BAD_ARG;
  std::ifstream in(path, std::ios::binary);
  if (!in.good()) return GGEM_ERR_BAD_ARG;
  uint32_t id = 0, len = 0;
  if (!get_be32(in, &id) || !get_be32(in, &len) || id != kPetscVecClassId) return GGEM_ERR_BAD_ARG;
  if (n_read) *n_read = len;
  if (!v) return GGEM_OK;
  if (n_expected >= 0 && (int64_t)len != n_expected) return GGEM_ERR_BAD_ARG;
  for (uint32_t i = 0; i < len; ++i) {
    unsigned char c[8];
    if (!in.read(reinterpret_cast<char *>(c), 8)) return GGEM_ERR_BAD_ARG;
    uint64_t b = 0;
    for (int k = 0; k < 8; ++k) b = (b << 8) | c[k];
    std::memcpy(v + i, &b, 8);
  }
  return GGEM_OK;
}
