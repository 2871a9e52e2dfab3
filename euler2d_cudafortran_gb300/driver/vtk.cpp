// vtk.cpp -- VTK ImageData writer (saveVTK of serial_ref/m_run.f90:653-720).
#include "vtk.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

bool little_endian() {
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

// Variable names of serial_ref/m_constants.f90:38 (3 characters each).
const char* kNames[4] = {"rho", "  E", " mx", " my"};

template <typename Real>
double at(const void* data, int isize, int jsize, int i, int j, int v) {
  return (double)static_cast<const Real*>(data)[((size_t)v * jsize + j) * isize + i];
}

}  // namespace

std::string save_vtk(const std::string& dir, int iStep, const void* data, int nx, int ny, int es, bool ascii) {
  char name[64];
  std::snprintf(name, sizeof(name), "euler2d_%08d.vti", iStep);
  const std::string path = dir.empty() ? std::string(name) : dir + "/" + name;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return std::string();
  const int isize = nx + 4, jsize = ny + 4;
  const char* ftype = es == 8 ? "Float64" : "Float32";
  std::fprintf(f, "<?xml version=\"1.0\"?>\n");
  std::fprintf(f, "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"%s\">\n",
               little_endian() ? "LittleEndian" : "BigEndian");
  std::fprintf(f, "  <ImageData WholeExtent=\"%7d%7d%7d%7d%7d%7d\"", 1, nx + 1, 1, ny + 1, 1, 2);
  std::fprintf(f, " Origin=\"0 0 0\" Spacing=\"1 1 1\">\n");
  std::fprintf(f, "  <Piece Extent=\"%7d%7d%7d%7d%7d%7d\">\n", 1, nx + 1, 1, ny + 1, 1, 2);
  std::fprintf(f, "   <PointData>\n    </PointData>\n    <CellData>\n");
  const size_t nbytes = (size_t)nx * ny * es;
  if (!ascii && nbytes >= (size_t)0xffffffffu) {
    std::fclose(f);
    return std::string();
  }
  for (int v = 0; v < 4; ++v) {
    if (ascii) {
      std::fprintf(f, "    <DataArray type=\"%s\" Name=\"%s\" format=\"ascii\" >\n", ftype, kNames[v]);
      for (int j = 2; j < ny + 2; ++j) {
        for (int i = 2; i < nx + 2; ++i)
          std::fprintf(f, " %.17g", es == 8 ? at<double>(data, isize, jsize, i, j, v)
                                            : at<float>(data, isize, jsize, i, j, v));
        std::fprintf(f, "\n");
      }
      std::fprintf(f, "    </DataArray>\n");
    } else {
      std::fprintf(f, "    <DataArray type=\"%s\" Name=\"%s\" format=\"appended\" offset=\"%zu\" />\n", ftype,
                   kNames[v], (size_t)v * (nbytes + 4));
    }
  }
  std::fprintf(f, "    </CellData>\n  </Piece>\n  </ImageData>\n");
  if (!ascii) {
    std::fprintf(f, "  <AppendedData encoding=\"raw\">\n   _");
    std::vector<unsigned char> row((size_t)nx * es);
    for (int v = 0; v < 4; ++v) {
      const uint32_t n = (uint32_t)nbytes;  // UInt32 block header (VTK's default header_type)
      std::fwrite(&n, sizeof(n), 1, f);
      for (int j = 2; j < ny + 2; ++j) {
        const unsigned char* src =
            static_cast<const unsigned char*>(data) + (((size_t)v * jsize + j) * isize + 2) * es;
        std::fwrite(src, 1, row.size(), f);
      }
    }
    std::fprintf(f, "\n  </AppendedData>\n");
  }
  std::fprintf(f, "</VTKFile>\n");
  std::fclose(f);
  return path;
}
