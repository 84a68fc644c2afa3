// VTK PolyData (.vtp) + ParaView collection (.pvd) output of a structured
// quad mesh, byte-compatible with the reference's PvdFileWriter2D
// (cppnabla/mesh/PvdFileWriter2D.cc:26-113, cppnabla/mesh/FileWriter.cc
// :20-35): same XML layout, same variable order (sorted names), numbers as
// the default C++ stream formats them (6 significant digits, %g style).
//
// Output is asynchronous: write() takes shared ownership of the dumped
// arrays and returns; a pool of formatting threads turns array chunks into
// text while one writer thread assembles the files in submission order, so
// the caller (the GPU loop) continues while earlier dumps are formatted.
// At most `max_pending` dumps are held in memory; write() waits beyond that.
#ifndef MAHYCO_GB300_PVD_WRITER_H
#define MAHYCO_GB300_PVD_WRITER_H

#include <condition_variable>
#include <cstddef>
#include <deque>
#include <functional>
#include <future>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

namespace hydro_out {

// Appends x as `std::ostream << x` with default flags writes it.
void append_g6(std::string& out, double x);
// Appends " v" for each of the n values (the writer's DataArray rows).
void append_values(std::string& out, const double* v, size_t n);

using Array = std::shared_ptr<const std::vector<double>>;
// name -> values; std::map keeps the reference's sorted-name order.
using Vars = std::map<std::string, Array>;

// Structured mesh of nx x ny quads of size dx x dy
// (cppnabla/mesh/CartesianMesh2DGenerator.cc:27-91): node (i, j) at
// (dx*i, dy*j), numbered row by row; quad (i, j) -> nodes
// (n, n+1, n+nx+2, n+nx+1) with n = j*(nx+1)+i.
struct Mesh {
  long nx = 0, ny = 0;
  double dx = 0.0, dy = 0.0;
  long nodes() const { return (nx + 1) * (ny + 1); }
  long cells() const { return nx * ny; }
};

class Writer;

// One module's output files (VnrRemap.*, EucclhydRemap.*, Particules.*) in
// a directory: FileWriter + PvdFileWriter2D.
class PvdSeries {
 public:
  // base "" -> "output"; "none"/"NONE" -> disabled; else base + "/output".
  // Creating a series empties its directory, as the reference does.  A null
  // mesh gives files with no points and no polygons that still list the
  // variable names (the reference's particle file, whose particle count is
  // zero).
  PvdSeries(Writer& w, std::string module, const std::string& base, const Mesh* mesh);
  bool disabled() const { return disabled_; }
  const std::string& directory() const { return dir_; }
  // Queues <module>.<iteration>.vtp and the rewrite of <module>.pvd.  Cell
  // arrays hold mesh->cells() values, node arrays mesh->nodes().  `xy`, when
  // given, holds the node positions of a mesh that moves (x, y per node, in
  // node order) in place of the generated mesh's.
  void write(int iteration, double time, const Vars& cell_vars, const Vars& node_vars,
             const Array& xy = nullptr);

 private:
  Writer& w_;
  std::string module_, dir_;
  bool disabled_ = false;
  long n_points_ = 0, n_cells_ = 0;
  std::map<double, std::string> files_by_time_;
  std::shared_future<std::string> points_, polys_;  // formatted once
};

class Writer {
 public:
  explicit Writer(int format_threads = 0, int max_pending = 2);
  ~Writer();  // waits for every queued file
  void flush();
  // first I/O error, empty if none
  std::string error();

 private:
  friend class PvdSeries;
  using Piece = std::shared_future<std::string>;
  struct File {
    std::string path;
    std::vector<Piece> pieces;
  };
  Piece text(std::string s);
  Piece format(std::function<std::string()> f);
  void submit(std::vector<File> files);
  void format_loop();
  void write_loop();

  std::mutex mu_;
  std::condition_variable cv_tasks_, cv_files_, cv_space_;
  std::deque<std::packaged_task<std::string()>> tasks_;
  std::deque<std::vector<File>> dumps_;
  int pending_ = 0, max_pending_;
  bool stop_ = false;
  std::string error_;
  std::vector<std::thread> pool_;
  std::thread writer_;
};

}  // namespace hydro_out

#endif
