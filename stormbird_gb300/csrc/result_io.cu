// SimulationResult JSON / reduced CSV formatting and the asynchronous result writer.
#include <charconv>
#include <cmath>
#include <stdexcept>
#include <sys/stat.h>

#include "result_io.hpp"
#include "sb_kernels.h"

namespace sbhost {

namespace {

// serde_json number: shortest round-trip digits; non-finite values become null.
void json_num(std::string& s, double v) {
    if (!std::isfinite(v)) {
        s += "null";
        return;
    }
    char buf[64];
    auto r = std::to_chars(buf, buf + sizeof(buf), v);
    s.append(buf, r.ptr);
}

// Rust's Display for f64: shortest round-trip digits in positional notation; NaN, inf, -inf.
void display_num(std::string& s, double v) {
    if (std::isnan(v)) {
        s += "NaN";
        return;
    }
    if (std::isinf(v)) {
        s += v > 0 ? "inf" : "-inf";
        return;
    }
    char buf[512];
    auto r = std::to_chars(buf, buf + sizeof(buf), v, std::chars_format::fixed);
    s.append(buf, r.ptr);
}

void json_vec(std::string& s, const double* p) {
    s += "{\"x\":";
    json_num(s, p[0]);
    s += ",\"y\":";
    json_num(s, p[1]);
    s += ",\"z\":";
    json_num(s, p[2]);
    s += '}';
}

void json_vec_array(std::string& s, const double* p, int n) {
    s += '[';
    for (int i = 0; i < n; ++i) {
        if (i) s += ',';
        json_vec(s, p + 3 * i);
    }
    s += ']';
}

void json_num_array(std::string& s, const double* p, int n) {
    s += '[';
    for (int i = 0; i < n; ++i) {
        if (i) s += ',';
        json_num(s, p[i]);
    }
    s += ']';
}

const char* kComponents[6] = {"circulatory", "viscous_lift", "sectional_drag", "added_mass", "gyroscopic", "total"};

}  // namespace

std::string result_json(const ResultRecord& r) {
    const sbgpu::OutLayout L = sbgpu::OutLayout::make(r.N, r.S);
    const double* o = r.out.data();
    const char* cs = r.body ? "\"Body\"" : "\"Global\"";
    std::string s;
    s.reserve(static_cast<size_t>(r.N) * 1200 + 1024);
    s += "{\"time\":";
    json_num(s, r.time);
    s += ",\"ctrl_points\":";
    json_vec_array(s, o + L.ctrl, r.N);
    s += ",\"solver_input_ctrl_points_velocity\":";
    json_vec_array(s, o + L.felt, r.N);
    // SectionalForcesInput (forces_and_moments.rs:34-49, force_calculations.rs:322-360)
    s += ",\"force_input\":{\"circulation_strength\":";
    json_num_array(s, o + L.gamma, r.N);
    s += ",\"velocity\":";
    json_vec_array(s, o + L.fvel, r.N);
    s += ",\"angles_of_attack\":";
    json_num_array(s, o + L.aoa, r.N);
    s += ",\"acceleration\":";
    json_vec_array(s, o + L.acc, r.N);
    sbgpu::d3 w = r.motion.velocity_angular;
    if (r.body) w = sbgpu::to_body(w, r.motion.rotation);
    const double wv[3] = {w.x, w.y, w.z};
    s += ",\"rotation_velocity\":";
    json_vec(s, wv);
    s += ",\"coordinate_system\":";
    s += cs;
    // SectionalForces (forces_and_moments.rs:53-72)
    s += "},\"sectional_forces\":{";
    for (int c = 0; c < 6; ++c) {
        s += '"';
        s += kComponents[c];
        s += "\":";
        json_vec_array(s, o + L.sect + static_cast<long long>(c) * r.N * 3, r.N);
        s += ',';
    }
    s += "\"coordinate_system\":";
    s += cs;
    s += '}';
    // IntegratedValues per wing (forces_and_moments.rs:22-30)
    for (int m = 0; m < 2; ++m) {
        s += m == 0 ? ",\"integrated_forces\":[" : ",\"integrated_moments\":[";
        const double* base = o + (m == 0 ? L.intf : L.intm);
        for (int wing = 0; wing < r.S; ++wing) {
            if (wing) s += ',';
            s += '{';
            for (int c = 0; c < 6; ++c) {
                if (c) s += ',';
                s += '"';
                s += kComponents[c];
                s += "\":";
                json_vec(s, base + (static_cast<long long>(wing) * 6 + c) * 3);
            }
            s += '}';
        }
        s += ']';
    }
    s += ",\"input_power\":[";  // NoPower (line_force_model/input_power.rs:33-35)
    for (int wing = 0; wing < r.S; ++wing) s += wing ? ",0.0" : "0.0";
    s += "],\"iterations\":";
    s += std::to_string(static_cast<long long>(o[L.iterations]));
    s += ",\"residual\":";
    json_num(s, o[L.residual]);
    s += ",\"wing_indices\":[";
    for (int wing = 0; wing < r.S; ++wing) {
        if (wing) s += ',';
        s += "{\"start\":" + std::to_string(r.wings[wing].first) + ",\"end\":" + std::to_string(r.wings[wing].second) + "}";
    }
    // RigidBodyMotion (stormath/src/rigid_body_motion.rs:22-28)
    const sbgpu::d3 mv[4] = {r.motion.translation, r.motion.rotation, r.motion.velocity_linear,
                             r.motion.velocity_angular};
    const char* mn[4] = {"translation", "rotation", "velocity_linear", "velocity_angular"};
    s += "],\"rigid_body_motion\":{";
    for (int k = 0; k < 4; ++k) {
        const double v[3] = {mv[k].x, mv[k].y, mv[k].z};
        s += '"';
        s += mn[k];
        s += "\":";
        json_vec(s, v);
        s += ',';
    }
    // the line force model's motion keeps the default rotation type (line_force_model/builder/
    // mod.rs:107-108 never sets it)
    s += "\"rotation_type\":\"XYZ\"}}";
    return s;
}

// results/simulation.rs:168-205, including its "time, " separator (comma and space).
void result_csv(const ResultRecord& r, std::string& header, std::string& data) {
    const sbgpu::OutLayout L = sbgpu::OutLayout::make(r.N, r.S);
    const double* o = r.out.data();
    header = "time,";
    data.clear();
    display_num(data, r.time);
    data += ", ";
    const char axes[3] = {'x', 'y', 'z'};
    for (int w = 0; w < r.S; ++w) {
        const std::string i = std::to_string(w);
        for (int k = 0; k < 3; ++k) header += "force_" + i + "." + axes[k] + ",";
        for (int k = 0; k < 3; ++k) {
            header += "moment_" + i + "." + axes[k];
            if (!(k == 2 && w == r.S - 1)) header += ',';
        }
        const double* f = o + L.intf + (static_cast<long long>(w) * 6 + 5) * 3;
        const double* m = o + L.intm + (static_cast<long long>(w) * 6 + 5) * 3;
        for (int k = 0; k < 3; ++k) {
            display_num(data, f[k]);
            data += ',';
        }
        for (int k = 0; k < 3; ++k) {
            display_num(data, m[k]);
            if (!(k == 2 && w == r.S - 1)) data += ',';
        }
    }
}

ResultWriter::ResultWriter(const std::string& path, int format) : path_(path), format_(format) {
    if (format != kResultsJsonHistory && format != kResultsCsv) throw std::runtime_error("unknown result format");
    if (format == kResultsJsonHistory) {
        file_ = std::fopen(path.c_str(), "wb");
        if (!file_) throw std::runtime_error("cannot create " + path);
        std::fputs("[\n", file_);
    } else {
        struct stat st;
        const bool exists = ::stat(path.c_str(), &st) == 0;
        file_ = std::fopen(path.c_str(), "ab");
        if (!file_) throw std::runtime_error("cannot open " + path);
        first_ = !exists;  // the header goes first into a file this writer creates
    }
    thread_ = std::thread([this] { run(); });
}

ResultWriter::~ResultWriter() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_.notify_all();
    if (thread_.joinable()) thread_.join();
    if (file_) {
        if (format_ == kResultsJsonHistory) std::fputs("\n]\n", file_);
        std::fclose(file_);
    }
}

void ResultWriter::push(ResultRecord&& r) {
    {
        std::lock_guard<std::mutex> lk(mu_);
        queue_.push_back(std::move(r));
        ++pushed_;
    }
    cv_.notify_one();
}

bool ResultWriter::flush() {
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [this] { return written_ == pushed_; });
    if (file_) std::fflush(file_);
    return !failed_;
}

void ResultWriter::run() {
    for (;;) {
        ResultRecord r;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [this] { return stop_ || !queue_.empty(); });
            if (queue_.empty()) return;  // stop requested and nothing left
            r = std::move(queue_.front());
            queue_.pop_front();
        }
        bool ok = true;
        if (format_ == kResultsJsonHistory) {
            const std::string s = result_json(r);
            if (!first_) ok = std::fputs(",\n", file_) >= 0;
            ok = ok && std::fwrite(s.data(), 1, s.size(), file_) == s.size();
        } else {
            std::string header, data;
            result_csv(r, header, data);
            if (first_) ok = std::fprintf(file_, "%s\n", header.c_str()) >= 0;
            ok = ok && std::fprintf(file_, "%s\n", data.c_str()) >= 0;
        }
        first_ = false;
        {
            std::lock_guard<std::mutex> lk(mu_);
            failed_ = failed_ || !ok;
            ++written_;
        }
        done_cv_.notify_all();
    }
}

// export.rs:75-163: the same elements, attributes, tab indentation and order; numbers in
// Rust's Display format.
std::string wake_vtp(const WakeRecord& w) {
    const long long n_pts = static_cast<long long>(w.W + 1) * w.Np, n_faces = static_cast<long long>(w.W) * w.N;
    std::string s;
    s.reserve(static_cast<size_t>(n_pts) * 72 + static_cast<size_t>(n_faces) * 96 + 1024);
    s += "<?xml version=\"1.0\"?>\n";
    s += "<VTKFile type=\"PolyData\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    s += "\t<PolyData>\n";
    s += "\t\t<Piece NumberOfPoints=\"" + std::to_string(n_pts) +
         "\" NumberOfVerts=\"0\" NumberOfLines=\"0\" NumberOfStrips=\"0\" NumberOfPolys=\"" + std::to_string(n_faces) +
         "\">\n";
    s += "\t\t\t<Points>\n";
    s += "\t\t\t\t<DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n";
    for (long long i = 0; i < n_pts; ++i) {
        s += "\t\t\t\t\t";
        display_num(s, w.pts[3 * i]);
        s += ' ';
        display_num(s, w.pts[3 * i + 1]);
        s += ' ';
        display_num(s, w.pts[3 * i + 2]);
        s += '\n';
    }
    s += "\t\t\t\t</DataArray>\n";
    s += "\t\t\t</Points>\n";
    s += "\t\t\t<Polys>\n";
    s += "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n";
    // panel_point_indices (dynamic_wake/mod.rs:82-91): point (row, j + wing) of each corner
    for (long long f = 0; f < n_faces; ++f) {
        const long long row = f / w.N;
        const int j = static_cast<int>(f % w.N);
        const long long c = j + w.wing_of_line[j];
        const long long a = row * w.Np + c, b = (row + 1) * w.Np + c;
        s += "\t\t\t\t\t" + std::to_string(a) + " " + std::to_string(a + 1) + " " + std::to_string(b + 1) + " " +
             std::to_string(b) + "\n";
    }
    s += "\t\t\t\t</DataArray>\n";
    s += "\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n";
    for (long long f = 0; f < n_faces; ++f) s += "\t\t\t\t\t" + std::to_string((f + 1) * 4) + "\n";
    s += "\t\t\t\t</DataArray>\n";
    s += "\t\t\t</Polys>\n";
    s += "\t\t\t<CellData Scalars=\"strength\">\n";
    const char* names[2] = {"strength", "viscous_core_length"};
    const std::vector<double>* vals[2] = {&w.str, &w.core};
    for (int a = 0; a < 2; ++a) {
        s += "\t\t\t\t<DataArray type=\"Float32\" Name=\"";
        s += names[a];
        s += "\" format=\"ascii\">\n";
        for (long long f = 0; f < n_faces; ++f) {
            s += "\t\t\t\t\t";
            display_num(s, (*vals[a])[f]);
            s += '\n';
        }
        s += "\t\t\t\t</DataArray>\n";
    }
    s += "\t\t\t</CellData>\n";
    s += "\t\t</Piece>\n";
    s += "\t</PolyData>\n";
    s += "</VTKFile>\n";
    return s;
}

WakeFileWriter::WakeFileWriter() { thread_ = std::thread([this] { run(); }); }

WakeFileWriter::~WakeFileWriter() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_.notify_all();
    if (thread_.joinable()) thread_.join();
}

void WakeFileWriter::push(WakeRecord&& w) {
    {
        std::lock_guard<std::mutex> lk(mu_);
        queue_.push_back(std::move(w));
        ++pushed_;
    }
    cv_.notify_one();
}

bool WakeFileWriter::flush() {
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [this] { return written_ == pushed_; });
    return !failed_;
}

void WakeFileWriter::run() {
    for (;;) {
        WakeRecord w;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [this] { return stop_ || !queue_.empty(); });
            if (queue_.empty()) return;
            w = std::move(queue_.front());
            queue_.pop_front();
        }
        const std::string text = wake_vtp(w);
        bool ok = false;
        if (std::FILE* f = std::fopen(w.path.c_str(), "wb")) {
            ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
            ok = std::fclose(f) == 0 && ok;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            failed_ = failed_ || !ok;
            ++written_;
        }
        done_cv_.notify_all();
    }
}

}  // namespace sbhost
