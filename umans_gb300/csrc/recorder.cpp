#include "recorder.hpp"

#include <cerrno>
#include <cstdio>
#include <cstring>

#include <sys/stat.h>

namespace umans {

TrajWriter::TrajWriter(const std::string& dir, int format) : dir_(dir), format_(format)
{
	// CSVWriter::SetOutputDirectory (csvwriter.cpp:30-40): a trailing slash,
	// the directory created when absent
	if (dir_.empty() || dir_.back() != '/') dir_ += '/';
	if (mkdir(dir_.c_str(), 0777) != 0 && errno != EEXIST) err_ = "cannot create " + dir_ + ": " + std::strerror(errno);
	th_ = std::thread([this] { run(); });
}

TrajWriter::~TrajWriter()
{
	{
		std::lock_guard<std::mutex> g(mu_);
		quit_ = true;
	}
	cv_.notify_all();
	if (th_.joinable()) th_.join();
}

std::string TrajWriter::error()
{
	std::lock_guard<std::mutex> g(mu_);
	return err_;
}

void TrajWriter::push(int n, int steps, std::vector<int> ids, std::vector<double> times, const float* xy,
                      cudaEvent_t ready, std::atomic<int>* busy, int stride, int offset)
{
	{
		std::lock_guard<std::mutex> g(mu_);
		jobs_.push_back(Job{ n, steps, stride, offset, std::move(ids), std::move(times), xy, ready, busy });
		++pending_;
	}
	cv_.notify_all();
}

void TrajWriter::drain()
{
	std::unique_lock<std::mutex> g(mu_);
	cv_.wait(g, [this] { return pending_ == 0; });
}

void TrajWriter::run()
{
	for (;;) {
		Job j;
		{
			std::unique_lock<std::mutex> g(mu_);
			cv_.wait(g, [this] { return quit_ || !jobs_.empty(); });
			if (jobs_.empty()) return;   // quit with nothing left
			j = std::move(jobs_.front());
			jobs_.pop_front();
		}
		cudaEventSynchronize(j.ready);
		write(j);
		j.busy->fetch_sub(1);
		{
			std::lock_guard<std::mutex> g(mu_);
			--pending_;
		}
		cv_.notify_all();
	}
}

void TrajWriter::write(const Job& j)
{
	std::string err;
	if (format_ == BINARY) {
		FILE* f = std::fopen((dir_ + "trajectory.bin").c_str(), "ab");
		if (!f) err = "cannot open " + dir_ + "trajectory.bin";
		else {
			const int hdr[2] = { j.n, j.steps };
			std::fwrite("UMTR", 1, 4, f);
			std::fwrite(hdr, sizeof(int), 2, f);
			std::fwrite(j.ids.data(), sizeof(int), (size_t)j.n, f);
			std::fwrite(j.times.data(), sizeof(double), (size_t)j.steps, f);
			for (int s = 0; s < j.steps; ++s)
				std::fwrite(j.xy + ((size_t)s * j.stride + j.offset) * 2, sizeof(float), (size_t)j.n * 2, f);
			if (std::fclose(f) != 0) err = "write error in " + dir_ + "trajectory.bin";
		}
	} else {
		// CSVWriter::Flush (csvwriter.cpp:42-66): per agent, its lines appended
		std::vector<char> buf;
		for (int k = 0; k < j.n && err.empty(); ++k) {
			buf.clear();
			char line[96];
			for (int s = 0; s < j.steps; ++s) {
				const float* p = j.xy + ((size_t)s * j.stride + j.offset + k) * 2;
				const int m = std::snprintf(line, sizeof(line), "%.10g,%.9g,%.9g\n", j.times[s], (double)p[0],
				                            (double)p[1]);
				buf.insert(buf.end(), line, line + m);
			}
			const std::string name = dir_ + "output_" + std::to_string(j.ids[k]) + ".csv";
			FILE* f = std::fopen(name.c_str(), "ab");
			if (!f) { err = "cannot open " + name; break; }
			std::fwrite(buf.data(), 1, buf.size(), f);
			if (std::fclose(f) != 0) err = "write error in " + name;
		}
	}
	if (!err.empty()) {
		std::lock_guard<std::mutex> g(mu_);
		if (err_.empty()) err_ = err;
	}
}

}  // namespace umans
