// io.hpp -- CSV output, directories and wall timing for the drop-in API.
//
// Same names and output format as the reference's src/utils/io.hpp:14-57:
// Csv writes optional "# comment" lines and one header line, then rows of
// numbers at 10 significant digits (stream precision 10, default float
// format), appending without a new header when asked to; write_panels writes
// one row per panel; Timer measures wall seconds.
#pragma once
#include <chrono>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <initializer_list>
#include <string>
#include <vector>
#include "mesh.hpp"

namespace bem {

inline void ensure_dir(const std::string& d) { std::filesystem::create_directories(d); }

class Csv {
public:
    Csv(const std::string& path, const std::string& header, const std::vector<std::string>& comments = {},
        bool append = false) {
        const std::filesystem::path p(path);
        if (p.has_parent_path()) ensure_dir(p.parent_path().string());
        const bool had_file = std::filesystem::exists(p);
        file_.open(path, append ? std::ios::app : std::ios::trunc);
        file_.precision(10);
        if (append && had_file) return;
        for (const auto& c : comments) file_ << "# " << c << "\n";
        file_ << header << "\n";
    }
    void row(std::initializer_list<double> v) { row(std::vector<double>(v)); }
    void row(const std::vector<double>& v) {
        const char* sep = "";
        for (double x : v) {
            file_ << sep << x;
            sep = ",";
        }
        file_ << "\n";
        file_.flush();
    }

private:
    std::ofstream file_;
};

// geometry, tag, velocity and traction of every panel
inline void write_panels(const std::string& path, const Mesh& M, const std::vector<V3>& u, const std::vector<V3>& f) {
    Csv c(path, "cx,cy,cz,nx,ny,nz,area,tag,ux,uy,uz,fx,fy,fz");
    for (int p = 0; p < M.P(); ++p)
        c.row({M.centroid[p].x, M.centroid[p].y, M.centroid[p].z, M.normal[p].x, M.normal[p].y, M.normal[p].z,
               M.area[p], (double)M.tags[p], u[p].x, u[p].y, u[p].z, f[p].x, f[p].y, f[p].z});
}

struct Timer {
    std::chrono::steady_clock::time_point start = std::chrono::steady_clock::now();
    double seconds() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    }
};

}  // namespace bem
