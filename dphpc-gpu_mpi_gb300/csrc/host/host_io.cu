// host_io.cu — the host side of the device -> host request channel (see runtime/rt_hostio.cuh).
//
// Replaces the reference's host loop over DeviceToHostCommunicator::processIncomingMessages
// (gpu_libs/gpu_main/main.cu:293-301, tests/test_runner.cuh:66-74) and its libc dispatcher
// (gpu_libs/gpu_main/libc_processor.cu:15-84, which serves fseek/fflush/fclose/fwrite/fopen/fread/remove on
// shared FILE* positions).  Here one service thread per world consumes the ring in ticket order while any
// launch of the world runs (a graph replay or an asynchronous launch included), and file data is
// addressed by explicit offsets (pread / pwrite), so requests of different ranks never share a seek
// position.  The thread sleeps when the ring is idle (backoff up to 200 us).
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../runtime/rt_hostio.cuh"
#include "host_io.h"

using gpumpi::HostArg;
using gpumpi::HostIO;
using gpumpi::HostReq;
using gpumpi::HostResp;
using gpumpi::HostRun;

struct HostService {
    HostReq* ring = nullptr;  // host addresses of the mapped allocations
    HostResp* resp = nullptr;
    unsigned char* window = nullptr;
    size_t window_bytes = 0;
    int cap = 0;
    int nranks = 0;
    unsigned long long next = 0;  // next ticket to serve
    std::vector<int> fds;         // handle h >= 3 -> fds[h - 3] (-1 once closed)
    std::thread th;
    std::atomic<bool> stop{false};
};

namespace {

int open_flags(long long f) {
    int o = 0;
    if ((f & gpumpi::HIO_F_READ) && (f & gpumpi::HIO_F_WRITE)) o = O_RDWR;
    else if (f & gpumpi::HIO_F_WRITE) o = O_WRONLY;
    else o = O_RDONLY;
    if (f & gpumpi::HIO_F_CREATE) o |= O_CREAT;
    if (f & gpumpi::HIO_F_EXCL) o |= O_EXCL;
    if (f & gpumpi::HIO_F_TRUNC) o |= O_TRUNC;
    if (f & gpumpi::HIO_F_APPEND) o |= O_APPEND;
    return o | O_CLOEXEC;
}

// the NUL-terminated string at the start of a window (bounded by the window)
std::string window_string(const unsigned char* w, size_t cap) {
    size_t n = 0;
    while (n < cap && w[n]) n++;
    return std::string((const char*)w, n);
}

int handle_fd(HostService* s, long long h) {
    if (h == gpumpi::HIO_STDOUT) return 1;
    if (h == gpumpi::HIO_STDERR) return 2;
    if (h < 3 || h - 3 >= (long long)s->fds.size()) return -1;
    return s->fds[(size_t)(h - 3)];
}

// Writes to a standard stream go through stdio (ordered with the host process's own output).
long long stream_write(long long h, const void* p, size_t n) {
    FILE* f = h == gpumpi::HIO_STDOUT ? stdout : stderr;
    const size_t k = fwrite(p, 1, n, f);
    fflush(f);
    return (long long)k;
}

long long do_rw(HostService* s, const HostReq& r, unsigned char* win, bool write) {
    const int fd = handle_fd(s, r.a0);
    if (fd < 0) return -EBADF;
    const long long nruns = r.nruns;
    if (nruns < 0 || (size_t)nruns * sizeof(HostRun) > s->window_bytes || r.a1 < 0 ||
        (size_t)r.a1 > s->window_bytes)
        return -EINVAL;
    const HostRun* runs = (const HostRun*)win;
    unsigned char* data = win + r.a1;
    const size_t room = s->window_bytes - (size_t)r.a1;
    size_t pos = 0;
    for (long long k = 0; k < nruns; k++) {
        const HostRun run = runs[k];
        if (run.len < 0 || pos + (size_t)run.len > room) return -EINVAL;
        size_t done = 0;
        while (done < (size_t)run.len) {
            ssize_t got;
            const size_t want = (size_t)run.len - done;
            if (write && (r.a0 == gpumpi::HIO_STDOUT || r.a0 == gpumpi::HIO_STDERR)) {
                got = (ssize_t)stream_write(r.a0, data + pos + done, want);
            } else if (run.off < 0) {
                got = write ? ::write(fd, data + pos + done, want) : ::read(fd, data + pos + done, want);
            } else {
                got = write ? ::pwrite(fd, data + pos + done, want, (off_t)(run.off + done))
                            : ::pread(fd, data + pos + done, want, (off_t)(run.off + done));
            }
            if (got < 0) {
                if (errno == EINTR) continue;
                return pos + done > 0 ? (long long)(pos + done) : -errno;
            }
            if (got == 0) return (long long)(pos + done);  // end of file (reads)
            done += (size_t)got;
        }
        pos += (size_t)run.len;
    }
    return (long long)pos;
}

// printf with the host's own formatter: the device sent the format string and one HostArg per value the
// conversions consume, in order ('*' widths and precisions included).
// Formats a HIO_PRINTF / HIO_SPRINTF request (format string at the window's start, packed arguments at a1).
std::string format_request(HostService* s, const HostReq& r, const unsigned char* win) {
    const std::string fmt = window_string(win, s->window_bytes);
    if (r.a1 < 0 || (size_t)r.a1 > s->window_bytes) return std::string();
    const unsigned char* ap = win + r.a1;
    const unsigned char* end = win + s->window_bytes;
    long long left = r.a2;
    auto next_arg = [&](HostArg& a, std::string* str) -> bool {
        if (left <= 0 || ap + sizeof(HostArg) > end) return false;
        memcpy(&a, ap, sizeof(HostArg));
        ap += sizeof(HostArg);
        left--;
        if (a.kind == gpumpi::HIO_ARG_STR) {
            if (a.len < 0 || ap + a.len > end) return false;
            if (str) str->assign((const char*)ap, (size_t)a.len);
            ap += (a.len + 7) & ~7;
        }
        return true;
    };
    std::string out;
    char buf[512];
    for (size_t i = 0; i < fmt.size();) {
        if (fmt[i] != '%') {
            out += fmt[i++];
            continue;
        }
        if (i + 1 < fmt.size() && fmt[i + 1] == '%') {
            out += '%';
            i += 2;
            continue;
        }
        // %[flags][width][.precision][length]conversion
        std::string spec = "%";
        size_t j = i + 1;
        while (j < fmt.size() && strchr("-+ #0", fmt[j])) spec += fmt[j++];
        auto take_num = [&](void) {
            if (j < fmt.size() && fmt[j] == '*') {
                HostArg a;
                if (next_arg(a, nullptr)) spec += std::to_string(a.v.i);
                j++;
            } else {
                while (j < fmt.size() && fmt[j] >= '0' && fmt[j] <= '9') spec += fmt[j++];
            }
        };
        take_num();
        if (j < fmt.size() && fmt[j] == '.') {
            spec += fmt[j++];
            take_num();
        }
        while (j < fmt.size() && strchr("hlLqjzt", fmt[j])) j++;  // the host applies its own length
        if (j >= fmt.size()) break;
        const char conv = fmt[j++];
        HostArg a{};
        std::string str;
        const bool have = next_arg(a, &str);
        int n = 0;
        switch (conv) {
        case 'd': case 'i':
            n = snprintf(buf, sizeof(buf), (spec + "lld").c_str(), have ? a.v.i : 0LL);
            break;
        case 'u': case 'x': case 'X': case 'o':
            n = snprintf(buf, sizeof(buf), (spec + "ll" + conv).c_str(), have ? a.v.u : 0ULL);
            break;
        case 'c':
            n = snprintf(buf, sizeof(buf), (spec + "c").c_str(), have ? (int)a.v.i : ' ');
            break;
        case 'f': case 'F': case 'e': case 'E': case 'g': case 'G': case 'a': case 'A':
            n = snprintf(buf, sizeof(buf), (spec + conv).c_str(), have ? a.v.d : 0.0);
            break;
        case 'p':
            n = snprintf(buf, sizeof(buf), (spec + "p").c_str(), have ? (void*)(uintptr_t)a.v.u : nullptr);
            break;
        case 's': {
            const int need = snprintf(nullptr, 0, (spec + "s").c_str(), str.c_str());
            if (need > 0) {
                std::vector<char> big((size_t)need + 1);
                snprintf(big.data(), big.size(), (spec + "s").c_str(), str.c_str());
                out.append(big.data(), (size_t)need);
            }
            n = 0;
            break;
        }
        default:
            out += spec;
            out += conv;
            n = 0;
        }
        if (n > 0) out.append(buf, (size_t)(n < (int)sizeof(buf) ? n : (int)sizeof(buf) - 1));
        i = j;
    }
    return out;
}

long long do_printf(HostService* s, const HostReq& r, const unsigned char* win) {
    if (r.a1 < 0 || (size_t)r.a1 > s->window_bytes) return -EINVAL;
    const std::string out = format_request(s, r, win);
    const long long h = r.a0;
    if (h == gpumpi::HIO_STDOUT || h == gpumpi::HIO_STDERR) return stream_write(h, out.data(), out.size());
    const int fd = handle_fd(s, h);
    if (fd < 0) return -EBADF;
    size_t done = 0;
    while (done < out.size()) {
        const ssize_t k = ::write(fd, out.data() + done, out.size() - done);
        if (k < 0) {
            if (errno == EINTR) continue;
            return -errno;
        }
        done += (size_t)k;
    }
    return (long long)out.size();
}

long long serve(HostService* s, const HostReq& r) {
    if (r.rank < 0 || r.rank >= s->nranks) return -EINVAL;
    unsigned char* win = s->window + (size_t)r.rank * s->window_bytes;
    switch (r.op) {
    case gpumpi::HIO_NOP: return 0;
    case gpumpi::HIO_OPEN: {
        const std::string path = window_string(win, s->window_bytes);
        const int fd = ::open(path.c_str(), open_flags(r.a0), 0644);
        if (fd < 0) return -errno;
        for (size_t k = 0; k < s->fds.size(); k++)
            if (s->fds[k] < 0) {
                s->fds[k] = fd;
                return (long long)k + 3;
            }
        s->fds.push_back(fd);
        return (long long)s->fds.size() + 2;
    }
    case gpumpi::HIO_CLOSE: {
        if (r.a0 < 3) return 0;  // standard streams stay open
        const int fd = handle_fd(s, r.a0);
        if (fd < 0) return -EBADF;
        s->fds[(size_t)(r.a0 - 3)] = -1;
        return ::close(fd) == 0 ? 0 : -errno;
    }
    case gpumpi::HIO_PWRITE: return do_rw(s, r, win, true);
    case gpumpi::HIO_PREAD: return do_rw(s, r, win, false);
    case gpumpi::HIO_SIZE: {
        const int fd = handle_fd(s, r.a0);
        struct stat st;
        if (fd < 0) return -EBADF;
        return fstat(fd, &st) == 0 ? (long long)st.st_size : -errno;
    }
    case gpumpi::HIO_REMOVE: {
        const std::string path = window_string(win, s->window_bytes);
        return ::unlink(path.c_str()) == 0 ? 0 : -errno;
    }
    case gpumpi::HIO_FLUSH: {
        if (r.a0 == gpumpi::HIO_STDOUT || r.a0 == gpumpi::HIO_STDERR) {
            fflush(r.a0 == gpumpi::HIO_STDOUT ? stdout : stderr);
            return 0;
        }
        const int fd = handle_fd(s, r.a0);
        if (fd < 0) return -EBADF;
        return fsync(fd) == 0 ? 0 : -errno;
    }
    case gpumpi::HIO_PRINTF: return do_printf(s, r, win);
    case gpumpi::HIO_SPRINTF: {
        if (r.a1 < 0 || (size_t)r.a1 > s->window_bytes) return -EINVAL;
        const std::string out = format_request(s, r, win);
        const size_t n = std::min(out.size(), s->window_bytes - 1);
        memcpy(win, out.data(), n);
        win[n] = 0;
        return (long long)out.size();
    }
    case gpumpi::HIO_TRUNCATE: {
        const int fd = handle_fd(s, r.a0);
        if (fd < 0) return -EBADF;
        return ftruncate(fd, (off_t)r.a1) == 0 ? 0 : -errno;
    }
    case gpumpi::HIO_GETENV: {
        const std::string name = window_string(win, s->window_bytes);
        const char* v = getenv(name.c_str());
        if (!v) return -ENOENT;
        const size_t n = std::min(strlen(v), s->window_bytes - 1);
        memcpy(win, v, n);
        win[n] = 0;
        return (long long)n;
    }
    default: return -ENOSYS;
    }
}

void service_loop(HostService* s) {
    unsigned idle = 0;
    while (!s->stop.load(std::memory_order_acquire)) {
        HostReq* slot = &s->ring[s->next & (unsigned long long)(s->cap - 1)];
        const unsigned long long seq = __atomic_load_n(&slot->seq, __ATOMIC_ACQUIRE);
        if (seq != s->next + 1) {
            // idle: spin briefly, then sleep with a growing interval (at most 200 us)
            if (++idle < 256) {
                std::this_thread::yield();
            } else {
                const unsigned us = idle < 1024 ? 20 : 200;
                std::this_thread::sleep_for(std::chrono::microseconds(us));
            }
            continue;
        }
        idle = 0;
        HostReq r;
        memcpy(&r, slot, sizeof(r));
        const long long res = serve(s, r);
        if (r.rank >= 0 && r.rank < s->nranks) {
            HostResp* rp = &s->resp[r.rank];
            rp->result = res;
            __atomic_store_n(&rp->answered, s->next + 1, __ATOMIC_RELEASE);
        }
        s->next++;
    }
}

template <class T>
cudaError_t mapped_alloc(T** host, T** dev, size_t bytes) {
    cudaError_t e = cudaHostAlloc((void**)host, bytes, cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) return e;
    memset(*host, 0, bytes);
    return cudaHostGetDevicePointer((void**)dev, *host, 0);
}

}  // namespace

HostService* hio_create(int nranks, size_t window_bytes, unsigned long long* d_tail, unsigned* d_broken, HostIO* desc,
                        std::string* err) {
    HostService* s = new HostService;
    s->nranks = nranks;
    s->window_bytes = window_bytes;
    int cap = 64;
    while (cap < nranks) cap *= 2;
    s->cap = cap;
    HostReq* d_ring = nullptr;
    HostResp* d_resp = nullptr;
    unsigned char* d_win = nullptr;
    cudaError_t e = mapped_alloc(&s->ring, &d_ring, sizeof(HostReq) * (size_t)cap);
    if (e == cudaSuccess) e = mapped_alloc(&s->resp, &d_resp, sizeof(HostResp) * (size_t)nranks);
    if (e == cudaSuccess) e = mapped_alloc(&s->window, &d_win, window_bytes * (size_t)nranks);
    if (e != cudaSuccess) {
        if (err) *err = std::string("host channel: ") + cudaGetErrorString(e);
        cudaGetLastError();
        hio_destroy(s);
        return nullptr;
    }
    desc->ring = d_ring;
    desc->resp = d_resp;
    desc->window = d_win;
    desc->tail = d_tail;
    desc->broken = d_broken;
    desc->window_bytes = (long long)window_bytes;
    desc->ring_cap = cap;
    s->th = std::thread(service_loop, s);
    return s;
}

void hio_destroy(HostService* s) {
    if (!s) return;
    s->stop.store(true, std::memory_order_release);
    if (s->th.joinable()) s->th.join();
    for (int fd : s->fds)
        if (fd >= 0) ::close(fd);
    if (s->ring) cudaFreeHost(s->ring);
    if (s->resp) cudaFreeHost(s->resp);
    if (s->window) cudaFreeHost(s->window);
    delete s;
}
