/**
 * @file Checkpoint.h
 * Particle checkpoints in the layout md-flexible writes and reads back
 * (examples/md-flexible/src/ParallelVtkWriter.cpp:55-200, MDFlexConfig.cpp:91-180): a VTK UnstructuredGrid with
 * the point data arrays velocities, forces, typeIds, ids and the points' positions, in that order, ASCII.
 * Values are written with max_digits10 significant digits so that reading a checkpoint restores the FP64
 * state exactly (md-flexible's own writer uses the stream's default precision); md-flexible's loader reads
 * either, because it only parses whitespace-separated numbers after each array name.
 */
#pragma once

#include <cstdint>
#include <fstream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace autopas_gb300 {

struct ParticleRecord {
  std::vector<double> x, y, z, vx, vy, vz, fx, fy, fz;
  std::vector<int64_t> typeId, id;
  size_t size() const { return x.size(); }
};

inline void writeRankRecord(const std::string &filename, const ParticleRecord &r) {
  std::ofstream f(filename, std::ios::out | std::ios::binary);
  if (!f.is_open()) throw std::runtime_error("writeRankRecord: cannot open " + filename);
  f.precision(std::numeric_limits<double>::max_digits10);
  const size_t n = r.size();
  f << "<?xml version=\"1.0\" encoding=\"UTF-8\" standalone=\"no\" ?>\n";
  f << "<VTKFile byte_order=\"LittleEndian\" type=\"UnstructuredGrid\" version=\"0.1\">\n";
  f << "  <UnstructuredGrid>\n";
  f << "    <Piece NumberOfCells=\"0\" NumberOfPoints=\"" << n << "\">\n";
  f << "      <PointData>\n";
  auto vec3 = [&](const char *name, const std::vector<double> &a, const std::vector<double> &b,
                  const std::vector<double> &c) {
    f << "        <DataArray Name=\"" << name << "\" NumberOfComponents=\"3\" format=\"ascii\" type=\"Float64\">\n";
    for (size_t i = 0; i < n; ++i) f << "        " << a[i] << " " << b[i] << " " << c[i] << "\n";
    f << "        </DataArray>\n";
  };
  auto scal = [&](const char *name, const std::vector<int64_t> &a) {
    f << "        <DataArray Name=\"" << name << "\" NumberOfComponents=\"1\" format=\"ascii\" type=\"Int64\">\n";
    for (size_t i = 0; i < n; ++i) f << "        " << a[i] << "\n";
    f << "        </DataArray>\n";
  };
  vec3("velocities", r.vx, r.vy, r.vz);
  vec3("forces", r.fx, r.fy, r.fz);
  scal("typeIds", r.typeId);
  scal("ids", r.id);
  f << "      </PointData>\n";
  f << "      <CellData/>\n";
  f << "      <Points>\n";
  vec3("positions", r.x, r.y, r.z);
  f << "      </Points>\n";
  f << "      <Cells>\n";
  f << "        <DataArray Name=\"types\" NumberOfComponents=\"0\" format=\"ascii\" type=\"Float32\"/>\n";
  f << "      </Cells>\n";
  f << "    </Piece>\n";
  f << "  </UnstructuredGrid>\n";
  f << "</VTKFile>\n";
  if (!f.good()) throw std::runtime_error("writeRankRecord: write failed for " + filename);
}

namespace detail {
inline void findWord(std::istream &in, const std::string &w) {
  std::string tok;
  while (in >> tok)
    if (tok.find(w) != std::string::npos) return;
  throw std::runtime_error("checkpoint: missing " + w);
}
}  // namespace detail

/** Reads a record written by writeRankRecord or by md-flexible (same order of arrays as MDFlexConfig.cpp:91-180). */
inline ParticleRecord readRankRecord(const std::string &filename) {
  std::ifstream in(filename);
  if (!in.is_open()) throw std::runtime_error("readRankRecord: cannot open " + filename);
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string text = ss.str();
  const auto p = text.find("NumberOfPoints=\"");
  if (p == std::string::npos) throw std::runtime_error("checkpoint: no NumberOfPoints");
  const size_t n = std::stoull(text.substr(p + 16));
  std::istringstream s(text);
  ParticleRecord r;
  auto read3 = [&](const char *name, std::vector<double> &a, std::vector<double> &b, std::vector<double> &c) {
    detail::findWord(s, std::string("Name=\"") + name + "\"");
    s.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
    a.resize(n);
    b.resize(n);
    c.resize(n);
    for (size_t i = 0; i < n; ++i) s >> a[i] >> b[i] >> c[i];
  };
  auto read1 = [&](const char *name, std::vector<int64_t> &a) {
    detail::findWord(s, std::string("Name=\"") + name + "\"");
    s.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
    a.resize(n);
    for (size_t i = 0; i < n; ++i) s >> a[i];
  };
  read3("velocities", r.vx, r.vy, r.vz);
  read3("forces", r.fx, r.fy, r.fz);
  read1("typeIds", r.typeId);
  read1("ids", r.id);
  read3("positions", r.x, r.y, r.z);
  if (!s) throw std::runtime_error("checkpoint: truncated " + filename);
  return r;
}

}  // namespace autopas_gb300
