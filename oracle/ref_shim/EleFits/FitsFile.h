// No-op stand-in for the EleFits FITS library, used only so that the
// reference renderer's Camera.cpp compiles for the oracle build. FITS output
// is never called by the oracle; every type here does nothing.
#pragma once
#include <string>
#include <vector>
#include <utility>
namespace Euclid {
namespace Cfitsio {
struct CfitsioError {};
}  // namespace Cfitsio
namespace Fits {
enum class FileMode { Read, Edit, Create, Overwrite, Temporary };
template <typename T>
struct Record {
  Record(std::string, T, std::string, std::string) {}
};
template <typename T>
struct Raster {
  std::vector<T> data;
};
template <typename T>
Raster<T> makeRaster(std::vector<T>&& v, long, long) {
  return Raster<T>{std::move(v)};
}
struct Header {
  template <typename... Ts>
  void writeSeq(const Ts&...) {}
};
struct SifFile {
  SifFile(const std::string&, FileMode) {}
  Header& header() { return h; }
  template <typename R, typename A>
  void write(const R&, const A&) {}
  Header h;
};
}  // namespace Fits
}  // namespace Euclid
