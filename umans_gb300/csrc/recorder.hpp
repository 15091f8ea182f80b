// Trajectory output: the GB300 counterpart of the reference's CSVWriter
// (src/Engine/tools/csvwriter.cpp:30-90, fed by CrowdSimulator::
// RunSimulationSteps, src/Engine/core/crowdSimulator.cpp:77-95).
//
// The engine keeps every step's positions in a device ring; a full ring is
// copied into page-locked host memory on the engine's stream and handed to
// this writer, whose thread waits for the copy and appends the chunk to the
// output while the GPU keeps stepping.
//
// Formats:
//  * CSV (the reference's layout): one file per agent, output_<id>.csv, one
//    "t,x,y" line per step appended; positions with 9 significant digits (every
//    float round-trips), times with 10;
//  * binary: one file trajectory.bin of appended chunks, each
//      "UMTR", int32 n, int32 steps, int32 ids[n], float64 times[steps],
//      float32 xy[steps][n][2]   (little-endian)
//    read back by umans_gb300.read_trajectory.
#pragma once
#include <atomic>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

namespace umans {

class TrajWriter {
public:
	enum Format { CSV = 0, BINARY = 1 };
	TrajWriter(const std::string& dir, int format);
	~TrajWriter();
	// error of the directory or of a write, empty when none
	std::string error();
	// Appends steps x n positions: agent k of step s at xy[(s * stride +
	// offset + k) * 2] (host memory valid once `ready` has completed; a batch
	// hands each scenario's writer its columns of one buffer).  *busy is
	// decremented when the writer no longer needs `xy`.
	void push(int n, int steps, std::vector<int> ids, std::vector<double> times, const float* xy,
	          cudaEvent_t ready, std::atomic<int>* busy, int stride, int offset);
	// waits until every chunk pushed so far is written
	void drain();

private:
	struct Job {
		int n, steps, stride, offset;
		std::vector<int> ids;
		std::vector<double> times;
		const float* xy;
		cudaEvent_t ready;
		std::atomic<int>* busy;
	};
	void run();
	void write(const Job& j);

	std::string dir_;
	int format_;
	std::thread th_;
	std::mutex mu_;
	std::condition_variable cv_;
	std::deque<Job> jobs_;
	int pending_ = 0;
	bool quit_ = false;
	std::string err_;
};

}  // namespace umans
