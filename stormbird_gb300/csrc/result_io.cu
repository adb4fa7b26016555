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

}  // namespace sbhost
