// Per-step results written out as the reference writes them: SimulationResult as JSON in
// serde's shape (stormbird/src/common_utils/results/simulation.rs:20-34, written by
// write_to_file, :91-98; a history file is a JSON array of them, result_history_from_file
// :37-45) and the reduced flattened CSV row (as_reduced_flatten_csv_string, :168-205, with
// the header written when the file is created, io_utils/csv_data.rs:11-33).
//
// ResultWriter formats and writes on its own thread from copies of the step's host output,
// so the next step's GPU work does not wait for the file system.
#pragma once

#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "sb_device.cuh"

namespace sbhost {

// One step's result: the library's output block (OutLayout) plus what SimulationResult
// carries besides it.
struct ResultRecord {
    double time = 0.0;
    int N = 0, S = 0;
    bool body = false;  // output coordinate system Body
    sbgpu::StepParams motion;
    std::vector<std::pair<int, int>> wings;  // line range of each wing
    std::vector<double> out;                 // OutLayout::make(N, S)
};

std::string result_json(const ResultRecord& r);
void result_csv(const ResultRecord& r, std::string& header, std::string& data);

enum ResultFormat : int { kResultsOff = 0, kResultsJsonHistory = 1, kResultsCsv = 2 };

class ResultWriter {
public:
    // Opens (JSON history: creates) the file; throws std::runtime_error when it cannot.
    ResultWriter(const std::string& path, int format);
    ~ResultWriter();  // writes what is queued, closes the JSON array, joins the thread
    void push(ResultRecord&& r);
    // Blocks until everything pushed so far is written; returns false after a write error.
    bool flush();

private:
    void run();
    std::string path_;
    int format_;
    std::FILE* file_ = nullptr;
    bool first_ = true;
    bool failed_ = false;
    bool stop_ = false;
    size_t pushed_ = 0, written_ = 0;
    std::deque<ResultRecord> queue_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::thread thread_;
};

// One step's dynamic wake for the VTK PolyData file the reference writes
// (lifting_line/wake/dynamic_wake/export.rs:75-163): points (streamwise-major rows of Np),
// quadrilateral panels (row-major, N per row) with their strength and viscous core length.
struct WakeRecord {
    std::string path;
    int N = 0, Np = 0, W = 0;
    std::vector<int> wing_of_line;  // [N]
    std::vector<double> pts;        // [(W + 1) Np][3]
    std::vector<double> str;        // [W N]
    std::vector<double> core;       // [W N]
};
std::string wake_vtp(const WakeRecord& w);

// Writes wake files on its own thread, one file per record, in push order.
class WakeFileWriter {
public:
    WakeFileWriter();
    ~WakeFileWriter();  // writes what is queued, joins the thread
    void push(WakeRecord&& w);
    bool flush();  // false after a write error

private:
    void run();
    bool failed_ = false, stop_ = false;
    size_t pushed_ = 0, written_ = 0;
    std::deque<WakeRecord> queue_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::thread thread_;
};

}  // namespace sbhost
