// rt_hostio.cuh — the device -> host request channel: ranks ask the host process to open, read, write,
// size, flush, close or remove files and to write formatted text to its standard streams.
//
// Replaces the reference's DeviceToHostCommunicator (gpu_libs/gpu_libc/cuda_mpi.cuh:392-435: a
// lock-protected circular queue in managed memory that the launcher's host loop polls,
// gpu_libs/gpu_main/main.cu:293-301, and serves with libc calls, gpu_libs/gpu_main/libc_processor.cu:15-84).
// Here nothing is locked and nothing migrates:
//   * the request ring, the per-rank response slots and the per-rank payload windows are page-locked host
//     memory that the GPU reaches in place (mapped); the host reads requests where the GPU wrote them;
//   * a rank claims a ring slot with one atomic on a device-memory ticket counter, fills it, and publishes
//     it with a system-scope release store of its sequence word; the host service thread consumes slots
//     strictly in ticket order and answers in the rank's own response slot (result, then a release store
//     of the answered ticket);
//   * a rank has at most one request outstanding (the call waits for its answer) and the ring has at least
//     as many slots as the world has ranks, so a claimed slot is always free: no wait for space, and every
//     claimed ticket is published;
//   * the rank's wait for the answer is bounded by the runtime timeout; a rank whose wait ran out marks
//     its channel broken (its window may still be written by a late answer) and its later calls fail.
// File data moves through the rank's payload window: writes are packed into it by the rank's block (the
// datatype map applied on the way), reads are unpacked from it; runs of (file offset, length) in the
// window describe where in the file each piece goes, so non-contiguous file views cost no extra pass.
#pragma once
#include <stdint.h>

namespace gpumpi {

// request operations
enum HostOp : int {
    HIO_NOP = 0,
    HIO_OPEN = 1,     // a0 = HIO_F_* flags; window: NUL-terminated path -> handle (>= 3) or -errno
    HIO_CLOSE = 2,    // a0 = handle -> 0 or -errno
    HIO_PWRITE = 3,   // a0 = handle, a1 = byte offset of the data in the window, nruns runs at window start
                      //   -> bytes written or -errno; a run offset of -1 appends at the stream's position
    HIO_PREAD = 4,    // as HIO_PWRITE, the host reads into the window -> bytes read (short at end of file)
    HIO_SIZE = 5,     // a0 = handle -> file size in bytes or -errno
    HIO_REMOVE = 6,   // window: NUL-terminated path -> 0 or -errno
    HIO_FLUSH = 7,    // a0 = handle: data reaches the file (fsync) or the stream is flushed -> 0 or -errno
    HIO_PRINTF = 8,   // a0 = handle; window: format string then packed arguments (HostArg) -> characters
    HIO_TRUNCATE = 9, // a0 = handle, a1 = size -> 0 or -errno
    HIO_GETENV = 10,  // window: NUL-terminated name -> the value, NUL-terminated, in the window: its length,
                      // or -ENOENT when the host process has no such variable
    HIO_SPRINTF = 11, // as HIO_PRINTF, the text is written into the window (NUL-terminated, cut to the
                      // window) instead of a stream -> its full length
};

// open flags (host maps them to open(2) flags)
enum : int {
    HIO_F_READ = 1,
    HIO_F_WRITE = 2,
    HIO_F_CREATE = 4,
    HIO_F_EXCL = 8,
    HIO_F_TRUNC = 16,
    HIO_F_APPEND = 32,
};

// handles of the host process's standard streams
constexpr int HIO_STDOUT = 1, HIO_STDERR = 2;

struct alignas(64) HostReq {
    unsigned long long seq;  // ticket + 1 once every other field is written (release, system scope)
    int op;
    int rank;
    long long a0, a1, a2;
    int nruns;
    int pad[3];
};

struct alignas(64) HostResp {
    unsigned long long answered;  // ticket + 1 once result (and any window data) is written (release)
    long long result;
    long long pad[6];
};

struct HostRun {  // one contiguous piece of a read or write: file byte offset and length
    long long off;
    long long len;
};

// packed printf argument: the device records each conversion's value by its C type; strings travel by
// content, right after their record
struct HostArg {
    int kind;   // HIO_ARG_*
    int len;    // string bytes (kind == HIO_ARG_STR), else 0
    union {
        long long i;
        unsigned long long u;
        double d;
    } v;
};
enum : int { HIO_ARG_INT = 1, HIO_ARG_UINT = 2, HIO_ARG_DOUBLE = 3, HIO_ARG_STR = 4, HIO_ARG_PTR = 5, HIO_ARG_CHAR = 6 };

// what the runtime descriptor holds about the channel (device addresses of the mapped host memory)
struct HostIO {
    HostReq* ring;                 // ring_cap slots (a power of two >= ranks)
    HostResp* resp;                // one per rank
    unsigned char* window;         // window_bytes per rank
    unsigned long long* tail;      // device memory: next ticket
    unsigned* broken;              // device memory, one per rank: a wait for the host ran out
    long long window_bytes;
    int ring_cap;
};

}  // namespace gpumpi
