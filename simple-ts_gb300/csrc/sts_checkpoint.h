// Checkpoint dumps of the solved fields in the reference's file format, written from a host
// thread while the next time steps run.
//
// Format (WriteSolvedDataToFile, SIMPLE_TS_MPI.cpp:5564-5731, and Write_it_ToFile,
// SIMPLE_TS_MPI.cpp:6742-6760): u, v, p and Temper as raw native-endian double[Nx*Ny]
// (`.bin`) or one `%.15e` value per line (`.txt`), vol_inf_fb as uint32[Nx*Ny], the time in
// it_begin.txt, the configuration in EnteredData.txt; with ToWriteSolvedDataToNewFiles a
// second copy of every dump carries the time in its name (u.<it>.bin ...).
//
// Pipeline of one save: the four fields are copied device-to-device into a snapshot buffer on
// the stepping stream (a few microseconds; the next step may then overwrite the fields), a
// second stream copies the snapshot into pinned host memory, and a writer thread waits for that
// copy and writes the files.  Two snapshot slots let one save be written while the next one is
// taken; a save waits only when both slots still hold unwritten dumps.  Saves are written in
// the order they were taken, so the last save of a file name wins, as in a serial run.
#pragma once
#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <deque>
#include <fstream>
#include <iomanip>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>

#include "sts_host.h"

namespace sts {

// Raw dump (WriteMassiveToBinaryFile, WriteReadData.h:107-136).  A file that cannot be opened
// is skipped: the reference does not check its stream either.
inline void write_bin(const std::string& f, const void* a, size_t bytes) {
  FILE* fp = std::fopen(f.c_str(), "wb");
  if (!fp) return;
  std::fwrite(a, 1, bytes, fp);
  std::fclose(fp);
}

// Text dump: one value per line in scientific notation with 15 digits (WriteMassiveToFile_1D,
// WriteReadData.h:139-170, as WriteSolvedDataToFile calls it).
template <class T>
void write_txt(const std::string& f, const T* a, size_t n) {
  std::ofstream o(f.c_str());
  for (size_t k = 0; k < n; k++) o << std::setiosflags(std::ios::scientific) << std::setprecision(15) << a[k] << "\n";
}

// The time as the reference streams a double (default ostream format), used in file names.
inline std::string num(double x) {
  std::ostringstream o;
  o << x;
  return o.str();
}

// What one save writes besides the four fields.
struct DumpSpec {
  std::string dir;           // case directory
  double it = 0;             // time of the save (it_begin.txt, per-save file names)
  bool bin = true, newf = false;
  Config cfg;                // EnteredData.txt as of the save
  const uint32_t* vol = nullptr;  // vol_inf_fb as the run keeps it (host; outlives the writer)
};

// Writes the files of one save from host copies of u, v, p, T (4 consecutive arrays of Na).
void write_dumps(const DumpSpec& d, const double* fields, size_t Na);

class Checkpointer {
 public:
  Checkpointer(int device, size_t Na) : device_(device), Na_(Na) {}
  ~Checkpointer();
  Checkpointer(const Checkpointer&) = delete;
  Checkpointer& operator=(const Checkpointer&) = delete;

  // Takes a snapshot of src[0..3] (u, v, p, T: device arrays of Na doubles, current on stream s)
  // and queues its files.  Returns 0 or an STS_ERR_* code with err set.
  int save(cudaStream_t s, const double* const src[4], DumpSpec spec, std::string& err);
  // Waits until every queued save is written; returns the first failure among them.
  int wait(std::string& err);

 private:
  struct Slot {
    double* dev = nullptr;   // 4*Na doubles on the device
    double* host = nullptr;  // 4*Na doubles, pinned
    cudaEvent_t copied = nullptr;
    bool busy = false;       // holds a save that is not written yet
  };
  struct Job {
    int slot;
    DumpSpec spec;
  };
  int init(std::string& err);
  void run();

  int device_;
  size_t Na_;
  bool ready_ = false;
  cudaStream_t copy_ = nullptr;
  cudaEvent_t snap_ = nullptr;
  Slot slot_[2];
  int next_ = 0;
  std::thread th_;
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<Job> q_;
  bool stop_ = false;
  std::string fail_;  // first failure of the writer thread
};

}  // namespace sts
