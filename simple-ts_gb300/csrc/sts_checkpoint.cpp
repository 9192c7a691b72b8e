// Checkpoint writer: snapshot on the stepping stream, copy on a second stream, files from a
// host thread (the pipeline is described in sts_checkpoint.h).
#include "sts_checkpoint.h"

#include <system_error>

#include "../../include/sts_gb300.h"

namespace sts {

// WriteSolvedDataToFile after its wall-temperature overwrite (SIMPLE_TS_MPI.cpp:5573-5692):
// the four fields and vol_inf_fb, the per-save copies under ToWriteSolvedDataToNewFiles
// (all five), then EnteredData.txt and it_begin.txt
// (WriteEnteredDataToFile, Write_it_ToFile, SIMPLE_TS_MPI.cpp:6742-6760).
void write_dumps(const DumpSpec& d, const double* fields, size_t Na) {
  static const char* names[4] = {"u", "v", "p", "Temper"};
  const std::string its = num(d.it);
  for (int k = 0; k < 4; k++) {
    const double* a = fields + (size_t)k * Na;
    const std::string base = d.dir + "/" + names[k];
    if (d.bin) {
      write_bin(base + ".bin", a, sizeof(double) * Na);
      if (d.newf) write_bin(base + "." + its + ".bin", a, sizeof(double) * Na);
    } else {
      write_txt(base + ".txt", a, Na);
      if (d.newf) write_txt(base + "." + its + ".txt", a, Na);
    }
  }
  if (d.bin) {
    write_bin(d.dir + "/vol_inf_fb.bin", d.vol, sizeof(uint32_t) * Na);
    if (d.newf) write_bin(d.dir + "/vol_inf_fb." + its + ".bin", d.vol, sizeof(uint32_t) * Na);
  } else {
    write_txt(d.dir + "/vol_inf_fb.txt", d.vol, Na);
    // the text per-save copy is named vol_inf_fb.txt.<it>.txt (SIMPLE_TS_MPI.cpp:5668)
    if (d.newf) write_txt(d.dir + "/vol_inf_fb.txt." + its + ".txt", d.vol, Na);
  }
  {
    std::ofstream itf((d.dir + "/it_begin.txt").c_str());
    itf << d.it << std::endl;
  }
  write_config(d.dir + "/EnteredData.txt", d.cfg);
}

namespace {
int cuda_fail(cudaError_t e, const char* what, std::string& err) {
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return STS_ERR_CUDA;
}
}  // namespace

#define CK(call)                                                \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call, err);    \
  } while (0)

// Buffers, copy stream and writer thread, made at the first save (a run that saves nothing
// holds none of them).  Memory: 2 slots x 4 fields x Na doubles on the device and as much pinned.
int Checkpointer::init(std::string& err) {
  const size_t bytes = 4 * Na_ * sizeof(double);
  CK(cudaStreamCreateWithFlags(&copy_, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&snap_, cudaEventDisableTiming));
  for (Slot& sl : slot_) {
    CK(cudaMalloc((void**)&sl.dev, bytes ? bytes : 8));
    CK(cudaMallocHost((void**)&sl.host, bytes ? bytes : 8));
    CK(cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming));
  }
  try {
    th_ = std::thread(&Checkpointer::run, this);
  } catch (const std::system_error& e) {
    err = std::string("cannot start the checkpoint writer thread: ") + e.what();
    return STS_ERR_CUDA;
  }
  ready_ = true;
  return STS_OK;
}

int Checkpointer::save(cudaStream_t s, const double* const src[4], DumpSpec spec, std::string& err) {
  if (!ready_) {
    if (int r = init(err)) return r;
  }
  const int k = next_;
  Slot& sl = slot_[k];
  {
    std::unique_lock<std::mutex> lk(m_);
    cv_.wait(lk, [&] { return !sl.busy; });
  }
  const size_t n = Na_ * sizeof(double);
  for (int f = 0; f < 4; f++) CK(cudaMemcpyAsync(sl.dev + (size_t)f * Na_, src[f], n, cudaMemcpyDeviceToDevice, s));
  CK(cudaEventRecord(snap_, s));
  CK(cudaStreamWaitEvent(copy_, snap_, 0));
  CK(cudaMemcpyAsync(sl.host, sl.dev, 4 * n, cudaMemcpyDeviceToHost, copy_));
  CK(cudaEventRecord(sl.copied, copy_));
  {
    std::lock_guard<std::mutex> lk(m_);
    sl.busy = true;
    q_.push_back(Job{k, std::move(spec)});
  }
  cv_.notify_all();
  next_ ^= 1;
  return STS_OK;
}

int Checkpointer::wait(std::string& err) {
  std::unique_lock<std::mutex> lk(m_);
  cv_.wait(lk, [&] { return q_.empty() && !slot_[0].busy && !slot_[1].busy; });
  if (!fail_.empty()) {
    err = fail_;
    fail_.clear();
    return STS_ERR_CUDA;
  }
  return STS_OK;
}

void Checkpointer::run() {
  cudaSetDevice(device_);
  for (;;) {
    Job j;
    {
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] { return stop_ || !q_.empty(); });
      if (q_.empty()) return;  // stopping, nothing left to write
      j = std::move(q_.front());
      q_.pop_front();
    }
    Slot& sl = slot_[j.slot];
    const cudaError_t e = cudaEventSynchronize(sl.copied);
    if (e == cudaSuccess) write_dumps(j.spec, sl.host, Na_);
    {
      std::lock_guard<std::mutex> lk(m_);
      if (e != cudaSuccess && fail_.empty())
        fail_ = std::string("checkpoint copy to the host failed: ") + cudaGetErrorString(e);
      sl.busy = false;
    }
    cv_.notify_all();
  }
}

Checkpointer::~Checkpointer() {
  if (th_.joinable()) {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    cv_.notify_all();
    th_.join();  // the queue is written out first
  }
  for (Slot& sl : slot_) {
    if (sl.copied) cudaEventDestroy(sl.copied);
    if (sl.host) cudaFreeHost(sl.host);
    if (sl.dev) cudaFree(sl.dev);
  }
  if (snap_) cudaEventDestroy(snap_);
  if (copy_) cudaStreamDestroy(copy_);
}

}  // namespace sts
