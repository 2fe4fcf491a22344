// mrc_io.cpp -- MRC tilt-series reader and volume writer, byte-compatible with the
// reference's MRCReader / MRCWriter (Code/MBIRLib/IOFilters/MRCReader.cpp:99-368,
// MRCWriter.cpp:90-290; header layout MRCHeader.h:46-212).  Fields are read and written at
// their fixed byte offsets, little-endian, so no struct packing is assumed.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#include "mbir_engine.h"

namespace mbir {

namespace {
constexpr int kHeaderBytes = 1024;
constexpr int kFeiBytes = 128;  // FEIHeader: 14 floats + 72 unused bytes

int32_t rd_i32(const unsigned char* b, int off) {
  int32_t v;
  std::memcpy(&v, b + off, 4);
  return v;
}
float rd_f32(const unsigned char* b, int off) {
  float v;
  std::memcpy(&v, b + off, 4);
  return v;
}
uint16_t rd_u16(const unsigned char* b) {
  uint16_t v;
  std::memcpy(&v, b, 2);
  return v;
}
void wr_i32(unsigned char* b, int off, int32_t v) { std::memcpy(b + off, &v, 4); }
void wr_f32(unsigned char* b, int off, float v) { std::memcpy(b + off, &v, 4); }
void wr_i16(unsigned char* b, int off, int16_t v) { std::memcpy(b + off, &v, 2); }
}  // namespace

int mrc_read(const std::string& path, const int* vmin, const int* vmax, MrcVolume& out,
             bool header_only, std::string& err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    err = "cannot open MRC file '" + path + "'";
    return MBIR_EIO;
  }
  unsigned char h[kHeaderBytes];
  if (std::fread(h, 1, kHeaderBytes, f) != kHeaderBytes) {
    std::fclose(f);
    err = "MRC header truncated";
    return MBIR_EIO;
  }
  out.nx = rd_i32(h, 0);
  out.ny = rd_i32(h, 4);
  out.nz = rd_i32(h, 8);
  out.mode = rd_i32(h, 12);
  const int32_t next = rd_i32(h, 92);
  if (out.nx <= 0 || out.ny <= 0 || out.nz <= 0 || next < 0) {
    std::fclose(f);
    err = "MRC header has invalid dimensions";
    return MBIR_EINVAL;
  }
  std::vector<unsigned char> ext(static_cast<size_t>(next));
  if (next > 0 && std::fread(ext.data(), 1, ext.size(), f) != ext.size()) {
    std::fclose(f);
    err = "MRC extended header truncated";
    return MBIR_EIO;
  }
  // FEI extended header is recognised by the first label (MRCReader.cpp:121-165)
  const std::string label0(reinterpret_cast<const char*>(h + 224), 80);
  out.has_fei = (label0.find("Fei Company") != std::string::npos ||
                 label0.find("EIC project") != std::string::npos ||
                 label0.find("MCAP project, MDG, Copyright 2013") != std::string::npos);
  if (label0.find("tif2mrc: Converted to MRC format") != std::string::npos) out.has_fei = false;
  out.a_tilt.clear();
  out.b_tilt.clear();
  out.pixel_size.clear();
  if (out.has_fei) {
    if (static_cast<int64_t>(next) < static_cast<int64_t>(kFeiBytes) * out.nz) {
      std::fclose(f);
      err = "FEI extended header shorter than nz entries";
      return MBIR_EINVAL;
    }
    for (int z = 0; z < out.nz; z++) {
      const unsigned char* e = ext.data() + static_cast<size_t>(z) * kFeiBytes;
      out.a_tilt.push_back(rd_f32(e, 0));
      out.b_tilt.push_back(rd_f32(e, 4));
      out.pixel_size.push_back(rd_f32(e, 44));
    }
  }
  if (header_only) {
    std::fclose(f);
    return MBIR_OK;
  }
  size_t tsize = 0;
  switch (out.mode) {
    case 0: tsize = 1; break;
    case 1: tsize = 2; break;
    case 2: tsize = 4; break;
    case 6: tsize = 2; break;
    default:
      std::fclose(f);
      err = "unsupported MRC mode";
      return MBIR_EINVAL;
  }
  int lo[3] = {0, 0, 0}, hi[3] = {out.nx - 1, out.ny - 1, out.nz - 1};
  if (vmin && vmax)
    for (int i = 0; i < 3; i++) {
      lo[i] = vmin[i];
      hi[i] = vmax[i];
    }
  const int dims[3] = {out.nx, out.ny, out.nz};
  for (int i = 0; i < 3; i++)
    if (lo[i] < 0 || hi[i] >= dims[i] || lo[i] > hi[i]) {
      std::fclose(f);
      err = "MRC sub-volume out of range";
      return MBIR_EINVAL;
    }
  const long data_start = kHeaderBytes + next;
  const int sx = hi[0] - lo[0] + 1, sy = hi[1] - lo[1] + 1, sz = hi[2] - lo[2] + 1;
  out.data.assign(static_cast<size_t>(sx) * sy * sz, 0.f);
  std::vector<unsigned char> row(static_cast<size_t>(sx) * tsize);
  size_t o = 0;
  // readPartialVolume (MRCReader.cpp:331-362): one x-run per (z, y)
  for (int z = lo[2]; z <= hi[2]; ++z)
    for (int y = lo[1]; y <= hi[1]; ++y) {
      const long long off = (static_cast<long long>(out.nx) * out.ny * z +
                             static_cast<long long>(out.nx) * y + lo[0]) *
                            static_cast<long long>(tsize);
      if (std::fseek(f, data_start + static_cast<long>(off), SEEK_SET) != 0 ||
          std::fread(row.data(), 1, row.size(), f) != row.size()) {
        std::fclose(f);
        err = "MRC data truncated";
        return MBIR_EIO;
      }
      for (int x = 0; x < sx; ++x) {
        float v;
        const unsigned char* p = row.data() + static_cast<size_t>(x) * tsize;
        switch (out.mode) {
          case 0: v = static_cast<float>(p[0]); break;
          case 1: {
            int16_t s;
            std::memcpy(&s, p, 2);
            v = static_cast<float>(s);
            break;
          }
          case 2: std::memcpy(&v, p, 4); break;
          default: {
            uint16_t s;
            std::memcpy(&s, p, 2);
            v = static_cast<float>(s);
            break;
          }
        }
        out.data[o++] = v;
      }
    }
  std::fclose(f);
  return MBIR_OK;
}

// MRCWriter::initializeMRCHeader + write (MRCWriter.cpp:90-290): float32 volume, sections
// written from z = N_z-1 down to 0, each section [y][x] over x in [x_start, x_end).
int mrc_write_volume(const std::string& path, const float* zxy, int n_z, int n_x, int n_y,
                     int x_start, int x_end, double length_x, std::string& err) {
  if (x_start < 0) x_start = 0;
  if (x_end > n_x) x_end = n_x;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    err = "cannot open '" + path + "' for writing";
    return MBIR_EIO;
  }
  unsigned char h[kHeaderBytes];
  std::memset(h, 0, sizeof(h));
  const int nx = x_end - x_start, ny = n_y, nz = n_z;
  wr_i32(h, 0, nx);
  wr_i32(h, 4, ny);
  wr_i32(h, 8, nz);
  wr_i32(h, 12, 2);
  wr_i32(h, 28, nx);
  wr_i32(h, 32, ny);
  wr_i32(h, 36, nz);
  wr_f32(h, 40, static_cast<float>(nx));
  wr_f32(h, 44, static_cast<float>(ny));
  wr_f32(h, 48, static_cast<float>(nz));
  wr_f32(h, 52, 90.f);
  wr_f32(h, 56, 90.f);
  wr_f32(h, 60, 90.f);
  wr_i32(h, 64, 1);
  wr_i32(h, 68, 2);
  wr_i32(h, 72, 3);
  wr_i16(h, 88, 0);
  wr_i32(h, 92, kFeiBytes * nz);
  std::memcpy(h + 208, "MAP ", 4);
  h[212] = 68;
  h[213] = 65;
  wr_i32(h, 220, 3);
  std::snprintf(reinterpret_cast<char*>(h + 224), 80, "Fei Company (C) Copyright 2003");
  std::snprintf(reinterpret_cast<char*>(h + 304), 80, "Reconstruction by OpenMBIR");
  std::snprintf(reinterpret_cast<char*>(h + 384), 80,
                "OpenMBIR code developed by Purdue University & BlueQuartz Software");
  std::fwrite(h, 1, kHeaderBytes, f);
  unsigned char fei[kFeiBytes];
  for (int i = 0; i < nz; ++i) {
    std::memset(fei, 0, sizeof(fei));
    wr_f32(fei, 44, static_cast<float>(length_x));
    std::fwrite(fei, 1, kFeiBytes, f);
  }
  std::vector<float> slice(static_cast<size_t>(nx) * ny);
  float mean = 0.0f;
  size_t count = 0;
  float dmax = static_cast<float>(std::numeric_limits<double>::min());
  float dmin = static_cast<float>(std::numeric_limits<double>::max());
  for (int z = n_z - 1; z >= 0; z--) {
    size_t idx = 0;
    for (int y = 0; y < ny; ++y)
      for (int x = x_start; x < x_end; ++x) {
        const float d = zxy[(static_cast<size_t>(z) * n_x + x) * n_y + y];
        slice[idx] = d;
        mean += slice[idx];
        count++;
        if (d > dmax) dmax = d;
        if (d < dmin) dmin = d;
        ++idx;
      }
    std::fwrite(slice.data(), sizeof(float), slice.size(), f);
  }
  mean = count ? mean / count : 0.f;
  std::fseek(f, 76, SEEK_SET);
  std::fwrite(&dmin, 4, 1, f);
  std::fwrite(&dmax, 4, 1, f);
  std::fwrite(&mean, 4, 1, f);
  std::fclose(f);
  return MBIR_OK;
}

// SigmaXEstimation::execute (GenericFilters/SigmaXEstimation.cpp:137-234): per view, the mean
// absolute deviation of the counts in a detector region (bright field: of log(counts +
// bf_offset), values <= 0 skipped in the sums but counted), divided by the target gain, times
// cos(tilt) / thickness, summed over the tilts and divided by the view count.  The region is read
// as the reference reads it, one reader per view (MRCReader.cpp:205-368): rows y0..y1 and columns
// x0..x1 inclusive, each run taken from the file at nx*ny*z + nx*y + x0 into one buffer of
// (x1-x0+1)(y1-y0+1) values, and the first (x1-x0)(y1-y0) values of the buffer used.  A run that
// starts at or past the end of the file reads nothing, one that crosses it keeps the bytes before
// it; either way that view's reading stops there and the estimate goes on with the next view
// (MRCReader::read returns success whatever its partial reads did).  The reference leaves the
// unread tail of its malloc'd buffer uninitialised; here it is zero.  That tail reaches the used
// values only when a default region (x1 = nx, y1 = ny) meets ny > nx + 1 on the last view.
// Unset bounds (< 0) are 0 and nx (ny).
int estimate_sigma_x(const std::string& path, double thickness, double target_gain,
                     bool use_bf_offset, double bf_offset, const float* tilts, int n_tilts,
                     const int* xd, const int* yd, double* out, std::string& err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    err = "cannot open MRC file '" + path + "'";
    return MBIR_EIO;
  }
  unsigned char h[kHeaderBytes];
  if (std::fread(h, 1, kHeaderBytes, f) != kHeaderBytes) {
    std::fclose(f);
    err = "MRC header truncated";
    return MBIR_EIO;
  }
  const int nx = rd_i32(h, 0), ny = rd_i32(h, 4), nz = rd_i32(h, 8), mode = rd_i32(h, 12);
  const int32_t next = rd_i32(h, 92);
  size_t ts = 0;
  switch (mode) {
    case 0: ts = 1; break;
    case 1: ts = 2; break;
    case 2: ts = 4; break;
    case 6: ts = 2; break;
    default: ts = 0;
  }
  if (nx <= 0 || ny <= 0 || nz <= 0 || next < 0 || ts == 0) {
    std::fclose(f);
    err = "MRC header: invalid dimensions or unsupported mode";
    return MBIR_EINVAL;
  }
  std::fseek(f, 0, SEEK_END);
  const long long file_bytes = std::ftell(f);
  const long long data_start = kHeaderBytes + static_cast<long long>(next);
  int x0 = xd ? xd[0] : -1, x1 = xd ? xd[1] : -1, y0 = yd ? yd[0] : -1, y1 = yd ? yd[1] : -1;
  if (x0 < 0) x0 = 0;
  if (x1 < 0) x1 = nx;
  if (y0 < 0) y0 = 0;
  if (y1 < 0) y1 = ny;
  const int32_t count = (x1 - x0) * (y1 - y0);
  const long long run = x1 - x0 + 1, rows = y1 - y0 + 1;
  std::vector<double> sum2s(static_cast<size_t>(nz), 0.0);
  const size_t n_values = (run > 0 && rows > 0) ? static_cast<size_t>(run * rows) : 0;
  std::vector<unsigned char> raw(n_values * ts);
  std::vector<double> buf(n_values);
  for (int z = 0; z < nz; ++z) {
    std::fill(raw.begin(), raw.end(), 0);
    size_t at = 0;  // bytes of the buffer filled so far
    for (int y = y0; y <= y1 && run > 0; ++y) {
      const long long off = data_start + (static_cast<long long>(nx) * ny * z +
                                          static_cast<long long>(nx) * y + x0) *
                                             static_cast<long long>(ts);
      const long long want = run * static_cast<long long>(ts);
      if (off < data_start || off >= file_bytes) break;  // peek() at the end of the file
      const long long got = std::min(want, file_bytes - off);
      std::fseek(f, static_cast<long>(off), SEEK_SET);
      if (std::fread(raw.data() + at, 1, static_cast<size_t>(got), f) !=
          static_cast<size_t>(got)) {
        std::fclose(f);
        err = "MRC read failed";
        return MBIR_EIO;
      }
      at += static_cast<size_t>(want);
      if (got != want) break;  // gcount() short of the run: the partial read stops the view
    }
    for (size_t i = 0; i < n_values; ++i) {
      const unsigned char* q = raw.data() + i * ts;
      double v = 0;
      if (mode == 0) v = q[0];
      if (mode == 1) v = static_cast<int16_t>(rd_u16(q));
      if (mode == 2) v = rd_f32(q, 0);
      if (mode == 6) v = rd_u16(q);
      buf[i] = v;
    }
    if (count <= 0 || static_cast<size_t>(count) > buf.size()) continue;
    double dev = 0, mean = 0;
    if (use_bf_offset) {  // calcBFAvgDeviation (:84-105)
      for (int32_t i = 0; i < count; i++) {
        const double t = buf[i] + bf_offset;
        if (t > 0) mean += std::log(t);
      }
      mean /= count;
      for (int32_t i = 0; i < count; i++) {
        const double t = buf[i] + bf_offset;
        if (t > 0) dev += std::fabs(std::log(t) - mean);
      }
    } else {  // calcAvgDeviation (:66-80)
      for (int32_t i = 0; i < count; i++) mean += buf[i];
      mean /= count;
      for (int32_t i = 0; i < count; i++) dev += std::fabs(buf[i] - mean);
    }
    dev /= count;
    sum2s[z] = dev;
  }
  std::fclose(f);
  double sum1 = 0.0;
  const float deg_to_rad = 0.017453292519943f;
  for (int i = 0; i < n_tilts && i < nz; ++i) {
    sum2s[i] /= target_gain;
    const double cosine = std::cos(tilts[i] * deg_to_rad);  // float cosine, as the reference
    sum1 += (sum2s[i] * cosine) / (thickness);
  }
  *out = sum1 / nz;
  return MBIR_OK;
}

// VTK legacy structured points, binary (VTKFileWriters.hpp:288-321 as writeVtkFile uses it,
// HAADF_ForwardModel.cpp:139-178): header lines, then the voxels as big-endian float32, z from
// the last slice down, y, x over [x_start, x_end).
int vtk_write_volume(const std::string& path, const float* zxy, int n_z, int n_x, int n_y,
                     int x_start, int x_end, std::string& err) {
  if (x_start < 0) x_start = 0;
  if (x_end > n_x) x_end = n_x;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    err = "cannot open '" + path + "' for writing";
    return MBIR_EIO;
  }
  const int nx = x_end - x_start;
  std::fprintf(f, "# vtk DataFile Version 2.0\n");
  std::fprintf(f, "data set from OpenMBIR\n");
  std::fprintf(f, "BINARY\n");
  std::fprintf(f, "DATASET STRUCTURED_POINTS\n");
  std::fprintf(f, "DIMENSIONS %d %d %d\n", nx, n_y, n_z);
  std::fprintf(f, "ORIGIN 0.0 0.0 0.0\n");
  std::fprintf(f, "SPACING %f %f %f\n", 1.0, 1.0, 1.0);
  std::fprintf(f, "POINT_DATA %d\n\n", nx * n_y * n_z);
  std::fprintf(f, "SCALARS %s float 1\n", "TomoVoxel");
  std::fprintf(f, "LOOKUP_TABLE default\n");
  std::vector<unsigned char> row(static_cast<size_t>(nx) * 4);
  for (int z = n_z - 1; z >= 0; z--)
    for (int y = 0; y < n_y; ++y) {
      for (int x = x_start; x < x_end; ++x) {
        uint32_t u;
        const float d = zxy[(static_cast<size_t>(z) * n_x + x) * n_y + y];
        std::memcpy(&u, &d, 4);
        unsigned char* o = row.data() + 4 * static_cast<size_t>(x - x_start);
        o[0] = static_cast<unsigned char>(u >> 24);
        o[1] = static_cast<unsigned char>(u >> 16);
        o[2] = static_cast<unsigned char>(u >> 8);
        o[3] = static_cast<unsigned char>(u);
      }
      std::fwrite(row.data(), 1, row.size(), f);
    }
  std::fclose(f);
  return MBIR_OK;
}

// AmiraMesh binary (AvizoUniformCoordinateWriter.cpp:110-196): text header with the lattice
// size, bounding box (voxel sizes delta_xy, delta_xy, delta_xz as float) and a float lattice,
// then "@1" and the voxels as little-endian float32, z from the last slice down, y, x.
int avizo_write_volume(const std::string& path, const float* zxy, int n_z, int n_x, int n_y,
                       int x_start, int x_end, double delta_xy, double delta_xz,
                       std::string& err) {
  if (x_start < 0) x_start = 0;
  if (x_end > n_x) x_end = n_x;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    err = "cannot open '" + path + "' for writing";
    return MBIR_EIO;
  }
  const size_t x = static_cast<size_t>(x_end - x_start), y = n_y, z = n_z;
  const float res[3] = {static_cast<float>(delta_xy), static_cast<float>(delta_xy),
                        static_cast<float>(delta_xz)};
  std::ostringstream ss;
  ss << "# AmiraMesh BINARY-LITTLE-ENDIAN 2.1\n\n";
  ss << "# Dimensions in x-, y-, and z-direction\n";
  ss << "define Lattice " << x << " " << y << " " << z << "\n\n";
  ss << "Parameters {\n";
  ss << "     OpenMBIRParams {\n";
  ss << "         Author \"OpenMBIR\",\n";
  ss << "         DateTime \"\"\n";
  ss << "     }\n";
  ss << "     Units {\n";
  ss << "         Coordinates \"microns\"\n";
  ss << "     }\n";
  ss << "     Content \"" << x << "x" << y << "x" << z << " int, uniform coordinates\",\n";
  const float o = 0.0f;
  ss << "     # Bounding Box is xmin xmax ymin ymax zmin zmax\n";
  ss << "     BoundingBox " << o << " " << o + (res[0] * x);
  ss << " " << o << " " << o + (res[1] * y);
  ss << " " << o << " " << o + (res[2] * z);
  ss << ",\n";
  ss << "     CoordType \"uniform\"\n";
  ss << "}\n\n";
  ss << "Lattice { float TomoVoxels } = @1\n\n";
  ss << "# Data section follows\n";
  ss << "@1\n";
  const std::string h = ss.str();
  std::fwrite(h.data(), 1, h.size(), f);
  std::vector<float> slice(x * y);
  for (int zz = n_z - 1; zz >= 0; zz--) {
    size_t idx = 0;
    for (int yy = 0; yy < n_y; ++yy)
      for (int xx = x_start; xx < x_end; ++xx)
        slice[idx++] = zxy[(static_cast<size_t>(zz) * n_x + xx) * n_y + yy];
    std::fwrite(slice.data(), sizeof(float), slice.size(), f);
  }
  std::fclose(f);
  return MBIR_OK;
}

// MRCSinogramInitializer::execute (MRCSinogramInitializer.cpp:79-339) plus the tilt read of
// the CLI (HAADFReconstructionArgsParser.cpp:296-322).
// The tilt series of an MRC file as MRCSinogramInitializer reads it (MRCSinogramInitializer.cpp:
// 113-300): the subvolume made symmetric about the centre of rotation and its y range a multiple
// of 3 x the interpolation factor, excluded views dropped; counts [theta][r][t].
int Engine::read_mrc_series(const char* path, std::vector<float>& counts,
                            std::vector<float>& tilts, int& n_theta_out, int& n_r_out,
                            int& n_t_out, double& dr_out, bool need_tilts) {
  if (!path) return fail(MBIR_EINVAL, "load_mrc: null path");
  MrcVolume hdr;
  std::string err;
  int rc = mrc_read(path, nullptr, nullptr, hdr, true, err);
  if (rc) return fail(rc, err);
  if (hdr.mode != 1 && hdr.mode != 2 && hdr.mode != 6)
    return fail(MBIR_EINVAL,
                "The data type of the MRC file was not either 1 (signed 16 Bit Ints), 2 (32 bit "
                "floats) or 6 (unsigned 16 Bit Ints)");
  if (need_tilts && !hdr.has_fei) return fail(MBIR_EINVAL, "MRC file carries no FEI tilt angles");
  int vmin[3] = {0, 0, 0}, vmax[3] = {hdr.nx - 1, hdr.ny - 1, hdr.nz - 1};
  if (p_.use_subvolume) {
    const int levels = p_.num_resolutions > 0 ? p_.num_resolutions : 1;
    const int interp = (1 << (levels - 1)) * (p_.final_resolution > 0 ? p_.final_resolution : 1);
    int xs = p_.subvolume[0], ys = p_.subvolume[1], zs = p_.subvolume[2];
    int xe = p_.subvolume[3], ye = p_.subvolume[4], ze = p_.subvolume[5];
    vmin[0] = xs;
    vmin[1] = ys;
    vmin[2] = zs;
    vmax[0] = xe;
    vmax[1] = ye;
    vmax[2] = ze;
    const double cor = hdr.nx / 2;  // integer division as in the reference
    double left = cor - vmin[0];
    double right = vmax[0] - cor + 1;
    if (left < 0) {
      vmin[0] = static_cast<int>(cor + left);
      left *= -1;
    }
    if (right < 0) {
      vmax[0] = static_cast<int>(cor - right);
      right *= -1;
    }
    if (left != right) {
      if (left < right) {
        double tx = cor + left - 1;
        if (tx >= hdr.nx) tx = hdr.nx - 1;
        vmax[0] = static_cast<int>(tx);
      } else {
        double tx = cor - right;
        if (tx < 0) tx = 0;
        vmin[0] = static_cast<int>(tx);
      }
    }
    const int16_t disty = static_cast<int16_t>(ye - ys + 1);
    const int16_t rem = static_cast<int16_t>(disty % (interp * 3));
    if (rem != 0) {
      const int16_t remainder = static_cast<int16_t>(interp * 3 - rem);
      if (ye + remainder < hdr.ny)
        ye += remainder;
      else
        ye = hdr.ny - 1;
    }
    vmax[1] = ye;
  }
  const int n_r = vmax[0] - vmin[0] + 1, n_t = vmax[1] - vmin[1] + 1;
  double dr = p_.default_pixel_size > 0 ? p_.default_pixel_size : 1.0;
  if (hdr.has_fei) dr = static_cast<double>(hdr.pixel_size[0]) * 1.0e9;
  std::vector<int> good;
  for (int i = vmin[2]; i <= vmax[2]; ++i) {
    bool keep = true;
    for (int j = 0; j < p_.n_excluded_views && j < 256; ++j)
      if (p_.excluded_views[j] == i) keep = false;
    if (keep) good.push_back(i);
  }
  if (good.empty()) return fail(MBIR_EINVAL, "no views left after exclusion");
  MrcVolume vol;
  rc = mrc_read(path, vmin, vmax, vol, false, err);
  if (rc) return fail(rc, err);
  const int n_theta = static_cast<int>(good.size());
  counts.assign(static_cast<size_t>(n_theta) * n_r * n_t, 0.f);
  tilts.assign(n_theta, 0.f);
  const std::vector<float>& src_tilts = p_.tilt_selection == 0 ? hdr.a_tilt : hdr.b_tilt;
  for (int z = 0; z < n_theta; z++) {
    const int dz = good[z] - vmin[2];
    // the reference indexes the tilt list by the kept-view position, not the file section
    // (MRCSinogramInitializer.cpp:271)
    if (z < static_cast<int>(src_tilts.size())) tilts[z] = src_tilts[z];
    for (int y = 0; y < n_t; y++)
      for (int x = 0; x < n_r; x++)
        counts[(static_cast<size_t>(z) * n_r + x) * n_t + y] =
            vol.data[static_cast<size_t>(dz) * n_r * n_t + static_cast<size_t>(y) * n_r + x];
  }
  n_theta_out = n_theta;
  n_r_out = n_r;
  n_t_out = n_t;
  dr_out = dr;
  return MBIR_OK;
}

int Engine::load_mrc(const char* path) {
  std::vector<float> counts, tilts;
  int n_theta = 0, n_r = 0, n_t = 0;
  double dr = 1.0;
  const int rc = read_mrc_series(path, counts, tilts, n_theta, n_r, n_t, dr, true);
  if (rc) return rc;
  return set_sinogram(counts.data(), tilts.data(), n_theta, n_r, n_t, dr, dr);
}

// The bright-field file of an HAADF reconstruction (initializeBrightFieldData,
// HAADF_ReconstructionEngine_Extra.cpp:84-149): read with the HAADF series' subvolume; when
// that read fails, once more over the HAADF sinogram's own extent; the sizes must then match.
int Engine::load_bright_field_mrc(const char* path) {
  if (state_ < 1) return fail(MBIR_ESTATE, "load_bright_field_mrc: set the sinogram first");
  std::vector<float> counts, tilts;
  int n_theta = 0, n_r = 0, n_t = 0;
  double dr = 1.0;
  int rc = read_mrc_series(path, counts, tilts, n_theta, n_r, n_t, dr, false);
  if (rc && rc != MBIR_EIO) {
    const mbir_params saved = p_;
    p_.use_subvolume = 1;
    p_.subvolume[0] = 0;
    p_.subvolume[1] = 0;
    p_.subvolume[2] = 0;
    p_.subvolume[3] = g_.n_r - 1;
    p_.subvolume[4] = g_.n_t - 1;
    p_.subvolume[5] = g_.n_theta - 1;
    rc = read_mrc_series(path, counts, tilts, n_theta, n_r, n_t, dr, false);
    p_ = saved;
  }
  if (rc) return rc;
  return set_bright_field(counts.data(), n_theta, n_r, n_t);
}

}  // namespace mbir
