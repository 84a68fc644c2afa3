// Asynchronous, byte-compatible VTK PolyData / PVD output (see pvd_writer.h).
#include "pvd_writer.h"

#include <algorithm>
#include <charconv>
#include <cstdio>
#include <filesystem>
#include <system_error>

namespace hydro_out {

namespace {

// values per formatting task: large arrays are cut so that several threads
// format one file
constexpr size_t kChunk = 1 << 17;

void append_int(std::string& out, long long v) {
  char buf[24];
  const auto r = std::to_chars(buf, buf + sizeof buf, v);
  out.append(buf, r.ptr);
}

}  // namespace

// std::ostream << double with default flags prints like printf("%.6g");
// std::to_chars in general format with precision 6 is specified to give the
// same characters (C++17 [utility.to.chars]), including "inf", "nan" and
// their signs.
void append_g6(std::string& out, double x) {
  char buf[40];
  const auto r = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::general, 6);
  out.append(buf, r.ptr);
}

void append_values(std::string& out, const double* v, size_t n) {
  out.reserve(out.size() + 14 * n);
  for (size_t i = 0; i < n; ++i) {
    out.push_back(' ');
    append_g6(out, v[i]);
  }
}

// ------------------------------------------------------------------ Writer
Writer::Writer(int format_threads, int max_pending)
    : max_pending_(max_pending < 1 ? 1 : max_pending) {
  int n = format_threads;
  if (n <= 0) {
    n = (int)std::thread::hardware_concurrency();
    if (n > 8) n = 8;
    if (n < 1) n = 1;
  }
  for (int i = 0; i < n; ++i) pool_.emplace_back([this] { format_loop(); });
  writer_ = std::thread([this] { write_loop(); });
}

Writer::~Writer() {
  flush();
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_tasks_.notify_all();
  cv_files_.notify_all();
  for (auto& t : pool_) t.join();
  writer_.join();
}

void Writer::flush() {
  std::unique_lock<std::mutex> lk(mu_);
  cv_space_.wait(lk, [this] { return pending_ == 0; });
}

std::string Writer::error() {
  std::lock_guard<std::mutex> lk(mu_);
  return error_;
}

Writer::Piece Writer::text(std::string s) {
  std::promise<std::string> p;
  p.set_value(std::move(s));
  return p.get_future().share();
}

Writer::Piece Writer::format(std::function<std::string()> f) {
  std::packaged_task<std::string()> task(std::move(f));
  Piece out = task.get_future().share();
  {
    std::lock_guard<std::mutex> lk(mu_);
    tasks_.push_back(std::move(task));
  }
  cv_tasks_.notify_one();
  return out;
}

void Writer::submit(std::vector<File> files) {
  std::unique_lock<std::mutex> lk(mu_);
  cv_space_.wait(lk, [this] { return pending_ < max_pending_; });
  ++pending_;
  dumps_.push_back(std::move(files));
  lk.unlock();
  cv_files_.notify_one();
}

void Writer::format_loop() {
  for (;;) {
    std::packaged_task<std::string()> task;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_tasks_.wait(lk, [this] { return stop_ || !tasks_.empty(); });
      if (tasks_.empty()) return;
      task = std::move(tasks_.front());
      tasks_.pop_front();
    }
    task();
  }
}

// Files are written in submission order, each from its pieces in order; a
// piece still being formatted is waited for here, never in a pool thread.
void Writer::write_loop() {
  for (;;) {
    std::vector<File> files;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_files_.wait(lk, [this] { return stop_ || !dumps_.empty(); });
      if (dumps_.empty()) return;
      files = std::move(dumps_.front());
      dumps_.pop_front();
    }
    std::string err;
    for (File& f : files) {
      FILE* fp = std::fopen(f.path.c_str(), "wb");
      if (!fp) {
        if (err.empty()) err = "cannot open " + f.path;
        for (Piece& p : f.pieces) p.wait();
        continue;
      }
      for (Piece& p : f.pieces) {
        const std::string& s = p.get();
        if (!s.empty() && std::fwrite(s.data(), 1, s.size(), fp) != s.size() && err.empty())
          err = "short write to " + f.path;
      }
      if (std::fclose(fp) != 0 && err.empty()) err = "cannot close " + f.path;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (error_.empty() && !err.empty()) error_ = err;
      --pending_;
    }
    cv_space_.notify_all();
  }
}

// --------------------------------------------------------------- PvdSeries
PvdSeries::PvdSeries(Writer& w, std::string module, const std::string& base, const Mesh* mesh)
    : w_(w), module_(std::move(module)) {
  namespace fs = std::filesystem;
  if (base.empty()) {
    dir_ = "output";
  } else if (base == "none" || base == "NONE") {
    disabled_ = true;
  } else {
    dir_ = base + "/output";
  }
  if (!disabled_) {
    std::error_code ec;
    if (fs::exists(dir_, ec)) fs::remove_all(dir_, ec);
    fs::create_directory(dir_, ec);
  }
  if (!mesh || disabled_) return;
  n_points_ = mesh->nodes();
  n_cells_ = mesh->cells();
  const Mesh m = *mesh;
  // node coordinates: " x y 0" per node (x = dx * i as a double product)
  points_ = w_.format([m] {
    std::string s;
    s.reserve((size_t)m.nodes() * 24);
    for (long j = 0; j <= m.ny; ++j)
      for (long i = 0; i <= m.nx; ++i) {
        s.push_back(' ');
        append_g6(s, m.dx * (double)(size_t)i);
        s.push_back(' ');
        append_g6(s, m.dy * (double)(size_t)j);
        s += " 0";
      }
    return s;
  });
  // connectivity rows "  a b c d", then the offsets " 4k"
  polys_ = w_.format([m] {
    std::string s;
    s.reserve((size_t)m.cells() * 40);
    const long nxn = m.nx + 1;
    for (long j = 0; j < m.ny; ++j)
      for (long i = 0; i < m.nx; ++i) {
        const long a = j * nxn + i, d = a + nxn;
        s += "  ";
        append_int(s, a);
        s.push_back(' ');
        append_int(s, a + 1);
        s.push_back(' ');
        append_int(s, d + 1);
        s.push_back(' ');
        append_int(s, d);
      }
    s += "\n\t\t\t\t</DataArray>\n\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n";
    for (long k = 1; k <= m.cells(); ++k) {
      s.push_back(' ');
      append_int(s, 4 * k);
    }
    return s;
  });
}

void PvdSeries::write(int iteration, double time, const Vars& cell_vars, const Vars& node_vars,
                      const Array& xy) {
  if (disabled_) return;
  std::vector<Writer::File> files(2);
  const std::string name = module_ + "." + std::to_string(iteration) + ".vtp";
  Writer::File& vtp = files[0];
  vtp.path = dir_ + "/" + name;
  std::string head =
      "<?xml version=\"1.0\"?>\n<VTKFile type=\"PolyData\">\n\t<PolyData>\n\t\t<Piece NumberOfPoints=\"";
  append_int(head, n_points_);
  head += "\" NumberOfPolys=\"";
  append_int(head, n_cells_);
  head += "\">\n\t\t\t<Points>\n\t\t\t\t<DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n";
  vtp.pieces.push_back(w_.text(std::move(head)));
  if (n_points_ && xy) {
    // a moving mesh: " x y 0" per node from this output's positions
    const long np = n_points_;
    Array keep = xy;
    vtp.pieces.push_back(w_.format([keep, np] {
      std::string s;
      s.reserve((size_t)np * 24);
      for (long q = 0; q < np; ++q) {
        s.push_back(' ');
        append_g6(s, (*keep)[2 * q]);
        s.push_back(' ');
        append_g6(s, (*keep)[2 * q + 1]);
        s += " 0";
      }
      return s;
    }));
  } else if (n_points_) {
    vtp.pieces.push_back(points_);
  }
  std::string mid =
      "\n\t\t\t\t</DataArray>\n\t\t\t</Points>\n\t\t\t<Polys>\n\t\t\t\t<DataArray type=\"Int32\" "
      "Name=\"connectivity\" format=\"ascii\">\n";
  if (n_cells_) {
    vtp.pieces.push_back(w_.text(std::move(mid)));
    vtp.pieces.push_back(polys_);
    mid.clear();
  } else {
    mid += "\n\t\t\t\t</DataArray>\n\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n";
  }
  mid += "\n\t\t\t\t</DataArray>\n\t\t\t</Polys>\n";
  vtp.pieces.push_back(w_.text(std::move(mid)));
  auto block = [&](const char* tag, const Vars& vars, long count) {
    if (vars.empty()) return;
    vtp.pieces.push_back(
        w_.text(std::string("\t\t\t<") + tag + " Scalars=\"" + vars.begin()->first + "\">\n"));
    for (const auto& [vname, arr] : vars) {
      vtp.pieces.push_back(
          w_.text("\t\t\t\t<DataArray Name=\"" + vname + "\" type=\"Float32\" format=\"ascii\">\n"));
      const long n = arr ? std::min(count, (long)arr->size()) : 0;
      for (long b = 0; b < n; b += (long)kChunk) {
        const long e = std::min(n, b + (long)kChunk);
        Array keep = arr;
        vtp.pieces.push_back(w_.format([keep, b, e] {
          std::string s;
          append_values(s, keep->data() + b, (size_t)(e - b));
          return s;
        }));
      }
      vtp.pieces.push_back(w_.text("\n\t\t\t\t</DataArray>\n"));
    }
    vtp.pieces.push_back(w_.text(std::string("\t\t\t</") + tag + ">\n"));
  };
  block("PointData", node_vars, n_points_);
  block("CellData", cell_vars, n_cells_);
  vtp.pieces.push_back(w_.text("\t\t</Piece>\n\t</PolyData>\n</VTKFile>\n"));

  files_by_time_[time] = name;
  Writer::File& pvd = files[1];
  pvd.path = dir_ + "/" + module_ + ".pvd";
  std::string s =
      "<?xml version=\"1.0\"?>\n<VTKFile type=\"Collection\" version=\"0.1\">\n\t<Collection>\n";
  for (const auto& [t, f] : files_by_time_) {
    s += "\t\t\t<DataSet timestep=\"";
    append_g6(s, t);
    s += "\" group=\"\" part=\"0\" file=\"" + f + "\"/>\n";
  }
  s += "\t</Collection>\n</VTKFile>\n";
  pvd.pieces.push_back(w_.text(std::move(s)));
  w_.submit(std::move(files));
}

}  // namespace hydro_out
