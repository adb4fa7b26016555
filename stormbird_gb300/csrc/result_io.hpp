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

}  // namespace sbhost
