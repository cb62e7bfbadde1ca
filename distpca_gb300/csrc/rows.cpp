// Host side of the block reader: where the packed SNP rows of a handle come from, and the ring of
// pinned staging slots that a reader thread fills ahead of the device.
//
// The reference reads each pass's SNP blocks from the .bed file with positional reads at
// 3 + ceil(n_ind/4) * start[j] (MPI_File_iread_at, methods.cpp:795-811, 873-874), overlapped
// with the previous block's decode and products.  Here a source hands out the rows of block j:
//   - file:   pread of the block's byte range from the .bed into a ring slot, by a reader thread
//             (split over several threads: one thread's pread from the page cache runs at memory-
//             copy speed, a few GB/s, below the host link);
//   - memory: caller rows in host memory, copied to the device in place (at full speed when
//             pinned; pageable rows take the driver's own staging);
//   - blocks: a caller callback that returns the host address of each block's rows (a
//             decompressor, a network receiver, a synthetic generator), treated like memory.
// The ring has kSlots slots of one block each.  Block i of a sweep goes to slot i % kSlots; the
// reader refills a slot once the host-to-device copy that read it (an event on the copy stream)
// has completed.  Every wait is bounded and reports DPCA_ERR_TIMEOUT; a short read reports
// DPCA_ERR_IO (the reference leaves MPI_File_iread_at's status unchecked, methods.cpp:803, 811).
#include <cuda_runtime.h>
#include <errno.h>
#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>

#include "dpca_internal.h"

namespace dpca {

namespace {
using Clock = std::chrono::steady_clock;
constexpr double kWaitSeconds = 120.0;   // a slot or a block that takes longer than this is an error
constexpr int kReadThreads = 8;          // threads per block read (file and pageable memory)
constexpr size_t kReadChunk = 64u << 20; // bytes per thread task

dpca_status pread_range(int fd, uint8_t *buf, size_t len, off_t off, const std::string &path, std::string *err) {
    while (len > 0) {
        ssize_t got = pread(fd, buf, len, off);
        if (got < 0 && errno == EINTR) continue;
        if (got <= 0) {
            char msg[512];
            snprintf(msg, sizeof(msg), "short read of %s at offset %lld (%s)", path.c_str(), (long long)off,
                     got < 0 ? strerror(errno) : "end of file");
            *err = msg;
            return DPCA_ERR_IO;
        }
        buf += got;
        off += got;
        len -= (size_t)got;
    }
    return DPCA_OK;
}

bool is_pinned(const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}
}  // namespace

RowSource::~RowSource() {
    if (fd >= 0) close(fd);
}

dpca_status RowSource::open_file(const char *bed_path, int64_t row_bytes) {
    kind = kFile;
    path = bed_path;
    np = row_bytes;
    header = 3;
    use_ring = true;
    fd = open(bed_path, O_RDONLY);
    if (fd < 0) {
        set_error("[Data::read_bed] Error reading file %s", bed_path);
        return DPCA_ERR_IO;
    }
    uint8_t magic[3] = {0, 0, 0};
    std::string err;
    if (pread_range(fd, magic, 3, 0, path, &err) != DPCA_OK || magic[0] != 0x6C || magic[1] != 0x1B ||
        magic[2] != 0x01) {
        set_error("%s is not a SNP-major PLINK .bed file", bed_path);
        return DPCA_ERR_FORMAT;
    }
    return DPCA_OK;
}

void RowSource::set_memory(const uint8_t *rows, int64_t row_stride, int64_t row_bytes) {
    kind = kMemory;
    base = rows;
    stride = row_stride;
    np = row_bytes;
    pinned = is_pinned(rows);
    use_ring = false;
}

void RowSource::set_blocks(dpca_block_fn f, void *c, int64_t row_bytes, int64_t max_row_stride) {
    kind = kBlocks;
    fn = f;
    ctx = c;
    np = row_bytes;
    max_stride = max_row_stride;
    use_ring = false;
}

// Rows [s0, s0 + rows) in place, when the source can hand them out without a copy.
dpca_status RowSource::direct(int64_t s0, int rows, const uint8_t **ptr, int64_t *row_stride, bool *pin) const {
    *ptr = nullptr;
    if (kind == kMemory) {
        *ptr = base + s0 * stride;
        *row_stride = stride;
        *pin = pinned;
        return DPCA_OK;
    }
    if (kind == kBlocks) {
        const uint8_t *p = nullptr;
        int64_t st = 0;
        int rc = fn(ctx, s0, rows, &p, &st);
        if (rc != 0 || !p || st < np || st > max_stride) {
            set_error("block source failed for rows [%lld, %lld) (status %d)", (long long)s0, (long long)s0 + rows, rc);
            return DPCA_ERR_IO;
        }
        *ptr = p;
        *row_stride = st;
        *pin = is_pinned(p);
        return DPCA_OK;
    }
    return DPCA_OK;  // file: never direct
}

// Rows [s0, s0 + rows) into dst (np bytes per row, contiguous), with several threads.
dpca_status RowSource::read_into(int64_t s0, int rows, uint8_t *dst, std::string *err) const {
    const uint8_t *src = nullptr;
    int64_t st = np;
    if (kind != kFile) {
        bool pin = false;
        dpca_status s = direct(s0, rows, &src, &st, &pin);
        if (s != DPCA_OK) {
            *err = "block source failed";
            return s;
        }
    }
    const size_t total = (size_t)rows * np;
    const int tasks = (int)std::min<size_t>(kReadThreads, std::max<size_t>(1, total / kReadChunk));
    dpca_status sts[kReadThreads];
    std::string errs[kReadThreads];
    auto work = [&](int t) {
        // task t: rows [r0, r1) of the block
        const int r0 = (int)((int64_t)rows * t / tasks), r1 = (int)((int64_t)rows * (t + 1) / tasks);
        sts[t] = DPCA_OK;
        if (kind == kFile) {
            sts[t] = pread_range(fd, dst + (size_t)r0 * np, (size_t)(r1 - r0) * np, (off_t)(header + (s0 + r0) * np),
                                 path, &errs[t]);
        } else if (st == np) {
            memcpy(dst + (size_t)r0 * np, src + (size_t)r0 * np, (size_t)(r1 - r0) * np);
        } else {
            for (int r = r0; r < r1; ++r) memcpy(dst + (size_t)r * np, src + (size_t)r * st, (size_t)np);
        }
    };
    if (tasks == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (int t = 1; t < tasks; ++t) th.emplace_back(work, t);
        work(0);
        for (auto &x : th) x.join();
    }
    for (int t = 0; t < tasks; ++t)
        if (sts[t] != DPCA_OK) {
            *err = errs[t].empty() ? "read failed" : errs[t];
            return sts[t];
        }
    return DPCA_OK;
}

// ------------------------------------------------------------------ ring
// Slot states: kFree (no data, no copy pending), kFilling (the reader writes it), kReady (holds
// block `block`, not yet taken), kInUse (taken: its copy is being enqueued), kReleased (its copy
// is enqueued; the buffer is free once the slot's event completes).
HostRing::~HostRing() { shutdown(); }

void HostRing::shutdown() {
    {
        std::lock_guard<std::mutex> lk(mu);
        stop = true;
    }
    cv.notify_all();
    if (reader.joinable()) reader.join();
    for (Slot &s : slots) {
        if (s.done) {
            cudaEventSynchronize(s.done);  // no copy may still read a slot that is freed
            cudaEventDestroy(s.done);
        }
        if (s.buf) cudaFreeHost(s.buf);
        s = Slot{};
    }
    slots.clear();
    slot_bytes = 0;
}

dpca_status HostRing::ensure(size_t bytes) {
    if (slot_bytes >= bytes && (int)slots.size() == kSlots) return DPCA_OK;
    shutdown();
    stop = false;
    slots.resize(kSlots);
    for (Slot &s : slots) {
        cudaError_t e = cudaHostAlloc((void **)&s.buf, std::max<size_t>(bytes, 1), cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("pinned staging ring: %zu bytes per slot: %s", bytes, cudaGetErrorString(e));
            shutdown();
            return DPCA_ERR_NOMEM;
        }
    }
    slot_bytes = bytes;
    reader = std::thread([this] { reader_main(); });
    return DPCA_OK;
}

// Start a sweep over `blocks` ({first row, rows} each) read from src.  The reader runs ahead of
// acquire() by up to kSlots blocks.  Blocks of an earlier sweep that were never taken are
// dropped; slots whose copies are still in flight are refilled only after those copies finish.
dpca_status HostRing::start(const RowSource *src, std::vector<std::pair<int64_t, int>> blocks) {
    size_t need = 0;
    for (auto &b : blocks) need = std::max(need, (size_t)b.second * (size_t)src->np);
    DPCA_TRY(ensure(need));
    {
        std::lock_guard<std::mutex> lk(mu);
        sweep_src = src;
        sweep = std::move(blocks);
        next_read = 0;
        ++generation;
        for (Slot &s : slots)
            if (s.state == kReady) s.state = kFree;
        failed = DPCA_OK;
        fail_msg.clear();
    }
    cv.notify_all();
    return DPCA_OK;
}

void HostRing::reader_main() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv.wait(lk, [&] { return stop || (sweep_src && next_read < (int)sweep.size() && failed == DPCA_OK); });
        if (stop) return;
        const int i = next_read;
        const uint64_t gen = generation;
        Slot &s = slots[i % kSlots];
        const auto t0 = Clock::now();
        // the slot's previous block must have been taken (its copy enqueued)
        const bool ok = cv.wait_for(lk, std::chrono::duration<double>(kWaitSeconds), [&] {
            return stop || generation != gen || s.state == kFree || s.state == kReleased;
        });
        if (stop) return;
        if (generation != gen) continue;
        if (!ok) {
            failed = DPCA_ERR_TIMEOUT;
            fail_msg = "staging ring: a slot was not released in time";
            cv.notify_all();
            continue;
        }
        const bool copy_pending = s.state == kReleased;
        s.state = kFilling;
        const auto blk = sweep[i];
        const RowSource *src = sweep_src;
        lk.unlock();
        dpca_status st = DPCA_OK;
        std::string err;
        if (copy_pending) {
            // the copy engine may still be reading this slot: poll its event (bounded)
            for (;;) {
                cudaError_t q = cudaEventQuery(s.done);
                if (q == cudaSuccess) break;
                if (q != cudaErrorNotReady) {
                    st = DPCA_ERR_CUDA;
                    err = std::string("staging ring: ") + cudaGetErrorString(q);
                    break;
                }
                if (std::chrono::duration<double>(Clock::now() - t0).count() > kWaitSeconds) {
                    st = DPCA_ERR_TIMEOUT;
                    err = "staging ring: a host-to-device copy did not finish in time";
                    break;
                }
                std::this_thread::sleep_for(std::chrono::microseconds(20));
            }
        }
        if (st == DPCA_OK) st = src->read_into(blk.first, blk.second, s.buf, &err);
        lk.lock();
        if (st != DPCA_OK && copy_pending && s.state == kFilling) {
            s.state = kReleased;  // the event is still the one to wait for
        } else {
            s.state = kFree;
        }
        if (generation != gen) {
            cv.notify_all();
            continue;
        }
        if (st != DPCA_OK) {
            failed = st;
            fail_msg = err;
        } else {
            s.state = kReady;
            s.block = i;
            next_read = i + 1;
        }
        cv.notify_all();
    }
}

dpca_status HostRing::acquire(int i, const uint8_t **ptr) {
    std::unique_lock<std::mutex> lk(mu);
    Slot &s = slots[i % kSlots];
    const bool ok = cv.wait_for(lk, std::chrono::duration<double>(kWaitSeconds),
                                [&] { return failed != DPCA_OK || (s.state == kReady && s.block == i); });
    if (failed != DPCA_OK) {
        set_error("%s", fail_msg.c_str());
        return failed;
    }
    if (!ok) {
        set_error("staging ring: block %d was not read in time", i);
        return DPCA_ERR_TIMEOUT;
    }
    s.state = kInUse;
    *ptr = s.buf;
    return DPCA_OK;
}

// The copy of block i out of its slot is enqueued on `stream`: record the slot's event there; the
// reader refills the slot once the event completes.
dpca_status HostRing::release(int i, cudaStream_t stream) {
    cudaError_t e;
    {
        std::lock_guard<std::mutex> lk(mu);
        Slot &s = slots[i % kSlots];
        e = cudaEventRecord(s.done, stream);
        s.state = kReleased;
    }
    cv.notify_all();
    if (e != cudaSuccess) {
        set_error("staging ring: %s", cudaGetErrorString(e));
        return DPCA_ERR_CUDA;
    }
    return DPCA_OK;
}

}  // namespace dpca
