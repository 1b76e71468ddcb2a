/*
 * p2m_pio.h -- positioned file reads of one contiguous range, split over several threads.
 * A single thread copying a large range from the page cache to user memory runs at one
 * core's memory rate (15 GB/s on the GB300 host: 26 ms for the 400 MB catalogue); each
 * thread here copies one contiguous part of the range (8 threads: 5 ms).  Used for the
 * catalogue read of the pks2map command line.  Writes into one file do not scale this
 * way (the file system serialises them), so there is no write counterpart.
 */
#ifndef P2M_PIO_H
#define P2M_PIO_H

#include <errno.h>
#include <unistd.h>

#include <algorithm>
#include <cstddef>
#include <thread>
#include <vector>

/* threads for one range: at most 8, and no more than the host offers */
inline int p2m_pio_threads() {
  const unsigned hc = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(8u, hc ? hc : 1u));
}

/* all of [off, off + bytes) of fd read into buf; parts of at least 1 MB, one per thread;
   false on an error or a short file */
inline bool p2m_pread_range(int fd, char *buf, size_t bytes, long long off, int threads) {
  const size_t mb = (size_t)1 << 20;
  size_t part = (bytes + (size_t)std::max(threads, 1) - 1) / (size_t)std::max(threads, 1);
  part = std::max(mb, (part + mb - 1) / mb * mb);
  const size_t nparts = bytes ? (bytes + part - 1) / part : 0;
  std::vector<char> ok(nparts, 0);
  auto run = [&](size_t i) {
    size_t done = i * part;
    const size_t end = std::min(bytes, done + part);
    while (done < end) {
      const ssize_t r = ::pread(fd, buf + done, end - done, (off_t)(off + (long long)done));
      if (r < 0 && errno == EINTR) continue;
      if (r <= 0) return;
      done += (size_t)r;
    }
    ok[i] = 1;
  };
  std::vector<std::thread> pool;
  for (size_t i = 1; i < nparts; i++) pool.emplace_back(run, i);
  if (nparts) run(0);
  for (auto &t : pool) t.join();
  return std::all_of(ok.begin(), ok.end(), [](char c) { return c != 0; });
}

inline bool p2m_pread_all(int fd, void *buf, size_t bytes, long long off) {
  return p2m_pread_range(fd, (char *)buf, bytes, off, p2m_pio_threads());
}

#endif /* P2M_PIO_H */
