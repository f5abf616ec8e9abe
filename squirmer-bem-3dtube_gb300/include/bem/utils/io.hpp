// io.hpp -- output files of the command-line modes (interface of
// src/utils/io.hpp: Csv, write_panels, ensure_dir, Timer).
//
// CSV file format, which downstream scripts and the stored reference outputs
// rely on:
//   * optional comment lines "# <text>", then one header line, then one line
//     per row: numbers separated by ',' without blanks, each printed with 10
//     significant digits in the shortest of fixed and scientific notation
//     ("%.10g": 0.04891121917, 1.0386961e-08, 4, nan);
//   * a file opened for appending that already exists gets rows only (no
//     comments, no header), so a resumed run continues its file;
//   * every row is flushed when written, so an interrupted run keeps its rows.
#pragma once
#include <chrono>
#include <cstdio>
#include <filesystem>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <vector>
#include "mesh.hpp"

namespace bem {

inline void ensure_dir(const std::string& dir) { std::filesystem::create_directories(dir); }

class Csv {
public:
    Csv(const std::string& path, const std::string& header, const std::vector<std::string>& comments = {},
        bool append = false) {
        const std::filesystem::path where(path);
        if (!where.parent_path().empty()) ensure_dir(where.parent_path().string());
        const bool continuing = append && std::filesystem::exists(where);
        fp_ = std::fopen(path.c_str(), append ? "a" : "w");
        if (!fp_) throw std::runtime_error("cannot write " + path);
        if (continuing) return;
        std::string head;
        for (const std::string& c : comments) head += "# " + c + "\n";
        head += header + "\n";
        std::fputs(head.c_str(), fp_);
    }
    Csv(const Csv&) = delete;
    Csv& operator=(const Csv&) = delete;
    ~Csv() {
        if (fp_) std::fclose(fp_);
    }

    void row(std::initializer_list<double> values) { emit(values.begin(), values.end()); }
    void row(const std::vector<double>& values) { emit(values.data(), values.data() + values.size()); }

private:
    std::FILE* fp_ = nullptr;

    void emit(const double* first, const double* last) {
        std::string line;
        char num[40];
        for (const double* v = first; v != last; ++v) {
            std::snprintf(num, sizeof num, "%.10g", *v);
            if (v != first) line += ',';
            line += num;
        }
        line += '\n';
        std::fputs(line.c_str(), fp_);
        std::fflush(fp_);
    }
};

// one row per panel: centroid, normal, area, tag, velocity, traction
inline void write_panels(const std::string& path, const Mesh& M, const std::vector<V3>& u, const std::vector<V3>& f) {
    Csv out(path, "cx,cy,cz,nx,ny,nz,area,tag,ux,uy,uz,fx,fy,fz");
    for (int p = 0; p < M.P(); ++p) {
        const V3 c = M.centroid[p], n = M.normal[p];
        out.row({c.x, c.y, c.z, n.x, n.y, n.z, M.area[p], (double)M.tags[p], u[p].x, u[p].y, u[p].z, f[p].x, f[p].y,
                 f[p].z});
    }
}

// wall-clock seconds since construction
struct Timer {
    std::chrono::steady_clock::time_point start = std::chrono::steady_clock::now();
    double seconds() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    }
};

}  // namespace bem
