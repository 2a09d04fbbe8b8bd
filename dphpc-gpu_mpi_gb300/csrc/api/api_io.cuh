// api_io.cuh — file and stream I/O from ranks, over the device -> host request channel
// (runtime/rt_hostio.cuh, served by host/host_io.cu).  Included by the runtime translation unit.
//
//  * gpumpi_* stdio (include/gpumpi_stdio.h.cuh): fopen/fclose/fwrite/fread/fputs/puts/fflush/remove and
//    fprintf/printf formatted by the host's own printf.  The reference's device libc returns nullptr
//    from fopen and traps in fclose/fputs/puts (gpu_libs/gpu_libc/stdio.cu:32-66) and prints through
//    CUDA's buffered device printf; these reach real files and the host's standard streams in call order.
//  * gpumpi_sprintf / snprintf / vsprintf / vsnprintf: formatted by the host into the rank's window.
//  * gpumpi_getenv (include/gpumpi_libc.h.cuh): the host process's environment.
//  * MPI-IO (MPI-3.1 chapter 13; the reference's gpu_libs/gpu_mpi/io.cu:139-559 and io.cuh:125-153):
//    collective open/close with the comm's rank 0 talking to the host, file views with any derived
//    filetype (positions are etypes of the view; a position maps to file byte disp + typemap(filetype,
//    position x etype size), so a non-contiguous view costs no extra pass), individual, explicit-offset
//    and shared file pointers, independent and collective (_all) data access.  Data is addressed by
//    explicit offsets on the host (pread/pwrite), so concurrent ranks never share a seek position (the
//    reference seeks one shared FILE* per request, io.cu:496-501).
// Deliberate differences from the reference: MPI_File is an opaque handle (the reference passes a struct
// by value); read/write calls return MPI_SUCCESS and report the amount in the status (the reference
// returns the element count, io.cu:474-509); MPI_File_delete is not collective (the reference adds a
// world barrier, io.cu:231-245); file pointers count etypes of the view (the reference mixes bytes and
// elements, io.cu:344-356,504).
#pragma once

namespace {

using gpumpi::HostArg;
using gpumpi::HostReq;
using gpumpi::HostResp;
using gpumpi::HostRun;

// ---- the channel ----
__device__ __forceinline__ unsigned long long ld_acquire_sys64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_sys64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned char* hio_window() {
    return c_rt.hio.window + (size_t)me() * (size_t)c_rt.hio.window_bytes;
}

constexpr long long HIO_EIO = -5, HIO_ENOSYS = -38, HIO_ETIMEDOUT = -110;

// Thread 0 of a rank: one request with the payload already in the rank's window; returns the host's
// answer (>= 0) or -errno.  The block's writes into the window were ordered before this call by the
// dispatch barrier; the system-scope fence makes them visible to the host before the release of `seq`.
__device__ __noinline__ long long host_call(int op, long long a0, long long a1, long long a2, int nruns) {
    const gpumpi::HostIO& h = c_rt.hio;
    if (!h.ring) return HIO_ENOSYS;
    const int r = me();
    if (ld_relaxed(&h.broken[r])) return HIO_EIO;
    const unsigned long long t = atomicAdd(h.tail, 1ULL);
    HostReq* q = &h.ring[t & (unsigned long long)(h.ring_cap - 1)];
    q->op = op;
    q->rank = r;
    q->a0 = a0;
    q->a1 = a1;
    q->a2 = a2;
    q->nruns = nruns;
    __threadfence_system();
    st_release_sys64(&q->seq, t + 1);
    Deadline d = make_deadline();
    while (ld_acquire_sys64(&h.resp[r].answered) != t + 1) {
        if (wait_tick(d, __LINE__, 4096)) {
            // the window may still be written by a late answer: this rank's channel stays closed
            atomicExch(&h.broken[r], 1u);
            return HIO_ETIMEDOUT;
        }
    }
    return *(volatile long long*)&h.resp[r].result;
}

// Copies the NUL-terminated string s into the window (truncated to the window); returns false if s is null.
__device__ bool window_put_string(const char* s) {
    if (!s || !c_rt.hio.ring) return false;  // a world made without the channel has no window
    unsigned char* w = hio_window();
    const long long cap = c_rt.hio.window_bytes;
    long long n = 0;
    while (n < cap - 1 && s[n]) {
        w[n] = (unsigned char)s[n];
        n++;
    }
    w[n] = 0;
    return true;
}

// Packed bytes [b0, b1) of (buf, t) to window bytes [0, b1 - b0) (to_window) or back; the rank's block
// copies (typed, the datatype map applied on the way) unless the buffer is thread 0's own memory.
__device__ void window_xfer(unsigned char* win, void* buf, const TypeDesc* t, long long b0, long long b1,
                            bool to_window) {
    if (b1 <= b0) return;
    const TypeDesc* tt = (t && !desc_contiguous(t)) ? t : nullptr;
    if (!tt) {
        if (to_window) t0_copy(win, nullptr, (const char*)buf + b0, nullptr, b1 - b0);
        else t0_copy((char*)buf + b0, nullptr, win, nullptr, b1 - b0);
        return;
    }
    if (!block_addressable(buf)) {
        if (to_window) typed_copy(win - b0, nullptr, buf, tt, b0, b1, 0, 1);
        else typed_copy(buf, tt, win - b0, nullptr, b0, b1, 0, 1);
        return;
    }
    Task task;
    task.kind = TASK_TYPED_COPY;
    task.n0 = b0;
    task.n1 = b1;
    if (to_window) {
        task.p0 = buf;
        task.p2 = tt;
        task.p1 = win - b0;
        task.p4 = nullptr;
    } else {
        task.p0 = win - b0;
        task.p2 = nullptr;
        task.p1 = buf;
        task.p4 = tt;
    }
    dispatch(task);
}

// ---- formatted output: the device records each conversion's argument, the host formats ----
__device__ long long put_arg(unsigned char* w, long long off, long long cap, int kind, long long iv, double dv,
                             const char* s) {
    if (off + (long long)sizeof(HostArg) > cap) return -1;
    HostArg a;
    a.kind = kind;
    a.len = 0;
    if (kind == gpumpi::HIO_ARG_DOUBLE) a.v.d = dv;
    else a.v.i = iv;
    long long n = 0;
    if (kind == gpumpi::HIO_ARG_STR) {
        const char* str = s ? s : "(null)";
        const long long room = cap - off - (long long)sizeof(HostArg);
        while (n < room && str[n]) n++;
        a.len = (int)n;
        for (long long k = 0; k < n; k++) w[off + (long long)sizeof(HostArg) + k] = (unsigned char)str[k];
    }
    memcpy(w + off, &a, sizeof(HostArg));
    return off + (long long)sizeof(HostArg) + ((n + 7) & ~7LL);
}

__device__ long long host_vformat(int op, long long handle, const char* fmt, va_list ap) {
    if (!fmt) return HIO_EIO;
    if (!c_rt.hio.ring) return HIO_ENOSYS;
    unsigned char* w = hio_window();
    const long long cap = c_rt.hio.window_bytes;
    long long flen = 0;
    while (flen < cap / 2 && fmt[flen]) {
        w[flen] = (unsigned char)fmt[flen];
        flen++;
    }
    w[flen] = 0;
    const long long a1 = (flen + 1 + 7) & ~7LL;
    long long off = a1, nargs = 0;
    for (long long i = 0; i < flen; i++) {
        if (fmt[i] != '%') continue;
        i++;
        if (i < flen && fmt[i] == '%') continue;
        while (i < flen && (fmt[i] == '-' || fmt[i] == '+' || fmt[i] == ' ' || fmt[i] == '#' || fmt[i] == '0')) i++;
        for (int part = 0; part < 2; part++) {  // width, then precision
            if (part == 1) {
                if (i < flen && fmt[i] == '.') i++;
                else break;
            }
            if (i < flen && fmt[i] == '*') {
                off = put_arg(w, off, cap, gpumpi::HIO_ARG_INT, va_arg(ap, int), 0.0, nullptr);
                nargs++;
                i++;
            } else {
                while (i < flen && fmt[i] >= '0' && fmt[i] <= '9') i++;
            }
            if (off < 0) break;
        }
        int lng = 0;  // 0 int, 1 long, 2 long long, -1 short/char (promoted to int)
        while (i < flen) {
            const char c = fmt[i];
            if (c == 'l') lng = lng >= 1 ? 2 : 1;
            else if (c == 'z' || c == 'j' || c == 't' || c == 'q') lng = 2;
            else if (c == 'h') lng = -1;
            else if (c != 'L') break;
            i++;
        }
        if (i >= flen || off < 0) break;
        const char conv = fmt[i];
        switch (conv) {
        case 'd': case 'i': {
            const long long v = lng >= 1 ? va_arg(ap, long long) : (long long)va_arg(ap, int);
            off = put_arg(w, off, cap, gpumpi::HIO_ARG_INT, v, 0.0, nullptr);
            break;
        }
        case 'u': case 'x': case 'X': case 'o': {
            const unsigned long long v =
                lng >= 1 ? va_arg(ap, unsigned long long) : (unsigned long long)va_arg(ap, unsigned);
            off = put_arg(w, off, cap, gpumpi::HIO_ARG_UINT, (long long)v, 0.0, nullptr);
            break;
        }
        case 'c': off = put_arg(w, off, cap, gpumpi::HIO_ARG_CHAR, va_arg(ap, int), 0.0, nullptr); break;
        case 'f': case 'F': case 'e': case 'E': case 'g': case 'G': case 'a': case 'A':
            off = put_arg(w, off, cap, gpumpi::HIO_ARG_DOUBLE, 0, va_arg(ap, double), nullptr);
            break;
        case 's': off = put_arg(w, off, cap, gpumpi::HIO_ARG_STR, 0, 0.0, va_arg(ap, const char*)); break;
        case 'p':
            off = put_arg(w, off, cap, gpumpi::HIO_ARG_PTR, (long long)(size_t)va_arg(ap, void*), 0.0, nullptr);
            break;
        case 'n': (void)va_arg(ap, void*); continue;  // nothing is written back
        default: continue;
        }
        nargs++;
    }
    if (off < 0) return HIO_EIO;
    return host_call(op, handle, a1, nargs, 0);
}
__device__ long long host_vprintf(long long handle, const char* fmt, va_list ap) {
    return host_vformat(gpumpi::HIO_PRINTF, handle, fmt, ap);
}

}  // namespace

// ------------------------------------------------------------------------------------------------
// gpumpi stdio
// ------------------------------------------------------------------------------------------------
__device__ gpumpi_FILE* gpumpi_fopen(const char* path, const char* mode) {
    if (!path || !mode) return nullptr;
    int f = 0;
    bool plus = false;
    for (const char* m = mode + 1; *m; m++) plus = plus || *m == '+';
    switch (mode[0]) {
    case 'r': f = gpumpi::HIO_F_READ | (plus ? gpumpi::HIO_F_WRITE : 0); break;
    case 'w': f = gpumpi::HIO_F_WRITE | gpumpi::HIO_F_CREATE | gpumpi::HIO_F_TRUNC | (plus ? gpumpi::HIO_F_READ : 0); break;
    case 'a': f = gpumpi::HIO_F_WRITE | gpumpi::HIO_F_CREATE | gpumpi::HIO_F_APPEND | (plus ? gpumpi::HIO_F_READ : 0); break;
    default: return nullptr;
    }
    for (const char* m = mode + 1; *m; m++)
        if (*m == 'x') f |= gpumpi::HIO_F_EXCL;
    window_put_string(path);
    const long long h = host_call(gpumpi::HIO_OPEN, f, 0, 0, 0);
    return h >= 3 ? (gpumpi_FILE*)(size_t)h : nullptr;
}

__device__ int gpumpi_fclose(gpumpi_FILE* f) {
    if (!f) return -1;
    return host_call(gpumpi::HIO_CLOSE, (long long)(size_t)f, 0, 0, 0) == 0 ? 0 : -1;
}

// Sequential transfer through the window in pieces of at most the window (less one run record).
__device__ long long stream_xfer(gpumpi_FILE* f, void* buf, long long bytes, bool write) {
    if (!f || !buf || bytes <= 0 || !c_rt.hio.ring) return 0;
    unsigned char* w = hio_window();
    const long long data_off = 16;
    const long long room = c_rt.hio.window_bytes - data_off;
    long long done = 0;
    while (done < bytes) {
        const long long n = bytes - done < room ? bytes - done : room;
        HostRun run;
        run.off = -1;
        run.len = n;
        if (write) window_xfer(w + data_off, (char*)buf + done, nullptr, 0, n, true);
        memcpy(w, &run, sizeof(run));
        const long long got =
            host_call(write ? gpumpi::HIO_PWRITE : gpumpi::HIO_PREAD, (long long)(size_t)f, data_off, 0, 1);
        if (got <= 0) break;
        if (!write) window_xfer(w + data_off, (char*)buf + done, nullptr, 0, got, false);
        done += got;
        if (got < n) break;
    }
    return done;
}

__device__ size_t gpumpi_fwrite(const void* ptr, size_t size, size_t nmemb, gpumpi_FILE* f) {
    if (size == 0 || nmemb == 0) return 0;
    return (size_t)(stream_xfer(f, (void*)ptr, (long long)(size * nmemb), true) / (long long)size);
}
__device__ size_t gpumpi_fread(void* ptr, size_t size, size_t nmemb, gpumpi_FILE* f) {
    if (size == 0 || nmemb == 0) return 0;
    return (size_t)(stream_xfer(f, ptr, (long long)(size * nmemb), false) / (long long)size);
}
__device__ int gpumpi_fputs(const char* s, gpumpi_FILE* f) {
    if (!s || !f) return -1;
    long long n = 0;
    while (s[n]) n++;
    return stream_xfer(f, (void*)s, n, true) == n ? 0 : -1;
}
__device__ int gpumpi_puts(const char* s) {
    if (gpumpi_fputs(s, gpumpi_stdout) < 0) return -1;
    const char nl = '\n';
    return stream_xfer(gpumpi_stdout, (void*)&nl, 1, true) == 1 ? 0 : -1;
}
__device__ int gpumpi_fflush(gpumpi_FILE* f) {
    if (!f) return 0;
    return host_call(gpumpi::HIO_FLUSH, (long long)(size_t)f, 0, 0, 0) == 0 ? 0 : -1;
}
__device__ int gpumpi_remove(const char* path) {
    if (!window_put_string(path)) return -1;
    return host_call(gpumpi::HIO_REMOVE, 0, 0, 0, 0) == 0 ? 0 : -1;
}
// sprintf family: the host formats (as for printf) into the rank's window; the text is copied to dst.  The
// result is cut to the window (host_window_bytes - 1 characters); the return value is the full length.
__device__ int gpumpi_vsnprintf(char* dst, size_t size, const char* fmt, va_list ap) {
    const long long n = host_vformat(gpumpi::HIO_SPRINTF, 0, fmt, ap);
    if (n < 0) {
        if (dst && size) dst[0] = 0;
        return -1;
    }
    if (dst && size) {
        const unsigned char* w = hio_window();
        long long m = n < c_rt.hio.window_bytes - 1 ? n : c_rt.hio.window_bytes - 1;
        if ((unsigned long long)m > size - 1) m = (long long)(size - 1);
        for (long long k = 0; k < m; k++) dst[k] = (char)w[k];
        dst[m] = 0;
    }
    return (int)n;
}
__device__ int gpumpi_vsprintf(char* dst, const char* fmt, va_list ap) {
    return gpumpi_vsnprintf(dst, ~(size_t)0, fmt, ap);
}
__device__ int gpumpi_snprintf(char* dst, size_t size, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    const int n = gpumpi_vsnprintf(dst, size, fmt, ap);
    va_end(ap);
    return n;
}
__device__ int gpumpi_sprintf(char* dst, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    const int n = gpumpi_vsnprintf(dst, ~(size_t)0, fmt, ap);
    va_end(ap);
    return n;
}
// The host process's environment variable `name`, or nullptr.  The value is copied into the calling
// rank's block (shared memory, at most 255 bytes) and stays valid until the rank's next gpumpi_getenv.
__shared__ char s_getenv_value[256];
__device__ char* gpumpi_getenv(const char* name) {
    if (!window_put_string(name)) return nullptr;
    const long long n = host_call(gpumpi::HIO_GETENV, 0, 0, 0, 0);
    if (n < 0) return nullptr;
    const unsigned char* w = hio_window();
    const long long m = n < 255 ? n : 255;
    for (long long k = 0; k < m; k++) s_getenv_value[k] = (char)w[k];
    s_getenv_value[m] = 0;
    return s_getenv_value;
}
__device__ int gpumpi_fprintf(gpumpi_FILE* f, const char* fmt, ...) {
    if (!f) return -1;
    va_list ap;
    va_start(ap, fmt);
    const long long n = host_vprintf((long long)(size_t)f, fmt, ap);
    va_end(ap);
    return n < 0 ? -1 : (int)n;
}
__device__ int gpumpi_printf(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    const long long n = host_vprintf(gpumpi::HIO_STDOUT, fmt, ap);
    va_end(ap);
    return n < 0 ? -1 : (int)n;
}

// ------------------------------------------------------------------------------------------------
// MPI-IO
// ------------------------------------------------------------------------------------------------
namespace {

constexpr unsigned FILE_MAGIC = 0x46494c45u;  // "FILE"

struct FileShared {                 // one per open file, made by the communicator's rank 0
    long long handle;               // host handle
    unsigned long long shared_pos;  // shared file pointer (etypes of the view), atomic
    int amode;
    char path[256];                 // for MPI_MODE_DELETE_ON_CLOSE
};

}  // namespace

struct MPI_File_impl {
    unsigned magic;
    FileShared* sh;
    MPI_Comm comm;
    int amode;
    long long disp;       // view displacement in bytes
    int etype, filetype;  // datatype handles of the view
    long long esize;      // etype size
    long long pos;        // individual file pointer, etypes of the view
    TypeDesc ft;          // the filetype's map, kept with the view (the handle may be freed)
    char datarep[16];
};

namespace {

__device__ __forceinline__ MPI_File_impl* check_file(MPI_File f) {
    return (f && f->magic == FILE_MAGIC) ? f : nullptr;
}

__device__ int errno_to_mpi(long long e) {
    switch (-e) {
    case 2: return GPUMPI_ERR_NO_SUCH_FILE;    // ENOENT
    case 17: return GPUMPI_ERR_FILE_EXISTS;    // EEXIST
    case 13: return GPUMPI_ERR_ACCESS;         // EACCES
    case 1: return GPUMPI_ERR_ACCESS;          // EPERM
    case 30: return GPUMPI_ERR_READ_ONLY;      // EROFS
    case 28: return GPUMPI_ERR_NO_SPACE;       // ENOSPC
    case 122: return GPUMPI_ERR_QUOTA;         // EDQUOT
    case 36: return GPUMPI_ERR_BAD_FILE;       // ENAMETOOLONG
    case 21: return GPUMPI_ERR_BAD_FILE;       // EISDIR
    default: return GPUMPI_ERR_IO;
    }
}

__device__ bool amode_ok(int amode) {
    const int acc = ((amode & MPI_MODE_RDONLY) ? 1 : 0) + ((amode & MPI_MODE_RDWR) ? 1 : 0) +
                    ((amode & MPI_MODE_WRONLY) ? 1 : 0);
    if (acc != 1) return false;
    if ((amode & MPI_MODE_RDONLY) && (amode & (MPI_MODE_CREATE | MPI_MODE_EXCL))) return false;
    if ((amode & MPI_MODE_RDWR) && (amode & MPI_MODE_SEQUENTIAL)) return false;
    return true;
}

__device__ void set_status(MPI_Status* st, long long bytes) {
    if (!st) return;
    st->MPI_SOURCE = MPI_ANY_SOURCE;
    st->MPI_TAG = MPI_ANY_TAG;
    st->MPI_ERROR = MPI_SUCCESS;
    st->count_bytes = bytes;
}

// Moves the packed bytes of (buf, count x dt) to or from the file at view position pos (etypes);
// returns the bytes moved (short only at the end of the file, for reads) or -errno.
__device__ long long file_xfer(MPI_File_impl* f, long long pos, void* buf, int count, MPI_Datatype dt, bool write) {
    const TypeDesc* ut = resolve_type(dt);
    if (!ut) return -22;
    const long long bytes = (long long)count * ut->size;
    if (bytes <= 0) return 0;
    const TypeDesc* ft = &f->ft;
    unsigned char* w = hio_window();
    const long long W = c_rt.hio.window_bytes;
    const int max_runs = W >= 16384 ? 256 : 16;
    const long long data_off = (long long)max_runs * (long long)sizeof(HostRun);
    const long long room = W - data_off;
    const long long q0 = pos * f->esize;  // packed offset in the view's filetype stream
    long long moved = 0;
    while (moved < bytes) {
        // the file runs of the next piece (merged where the filetype is contiguous across blocks)
        HostRun runs[8];
        int nruns = 0, staged = 0;
        long long q = q0 + moved;
        const long long q_end = q0 + moved + (bytes - moved < room ? bytes - moved : room);
        while (q < q_end && nruns < max_runs) {
            const long long qe = q % ft->size;
            long long len = ft->block - (qe % ft->block);
            if (len > q_end - q) len = q_end - q;
            const long long off = f->disp + desc_map(ft, q);
            HostRun* last = staged > 0 ? &runs[staged - 1] : nullptr;
            if (last && last->off + last->len == off) {
                last->len += len;
            } else {
                if (staged == 8) {  // flush the local batch of run records into the window
                    memcpy(w + (long long)(nruns - staged) * sizeof(HostRun), runs, sizeof(runs));
                    staged = 0;
                }
                runs[staged].off = off;
                runs[staged].len = len;
                staged++;
                nruns++;
            }
            q += len;
        }
        if (staged) memcpy(w + (long long)(nruns - staged) * sizeof(HostRun), runs, sizeof(HostRun) * staged);
        const long long n = q - (q0 + moved);
        if (write) window_xfer(w + data_off, buf, ut, moved, moved + n, true);
        const long long got =
            host_call(write ? gpumpi::HIO_PWRITE : gpumpi::HIO_PREAD, f->sh->handle, data_off, 0, nruns);
        if (got < 0) return moved > 0 ? moved : got;
        if (!write) window_xfer(w + data_off, buf, ut, moved, moved + got, false);
        moved += got;
        if (got < n) break;
    }
    return moved;
}

__device__ int io_check(MPI_File_impl* f, MPI_Datatype dt, int count, bool write) {
    if (!f) return GPUMPI_ERR_FILE;
    if (count < 0) return GPUMPI_ERR_COUNT;
    const TypeDesc* ut = resolve_type(dt);
    if (!ut) return GPUMPI_ERR_TYPE;
    if (((long long)count * ut->size) % f->esize) return GPUMPI_ERR_ARG;  // whole etypes only
    if (write && (f->amode & MPI_MODE_RDONLY)) return GPUMPI_ERR_READ_ONLY;
    if (!write && (f->amode & MPI_MODE_WRONLY)) return GPUMPI_ERR_AMODE;  // as the reference, io.cu:460
    return MPI_SUCCESS;
}

__device__ int io_at(MPI_File fh, MPI_Offset offset, void* buf, int count, MPI_Datatype dt, MPI_Status* st, bool write) {
    MPI_File_impl* f = check_file(fh);
    int rc = io_check(f, dt, count, write);
    if (rc) return rc;
    if (f->amode & MPI_MODE_SEQUENTIAL) return GPUMPI_ERR_UNSUPPORTED_OPERATION;
    if (offset < 0) return GPUMPI_ERR_ARG;
    const long long got = file_xfer(f, offset, buf, count, dt, write);
    if (got < 0) return errno_to_mpi(got);
    set_status(st, got);
    return MPI_SUCCESS;
}

__device__ int io_ind(MPI_File fh, void* buf, int count, MPI_Datatype dt, MPI_Status* st, bool write) {
    MPI_File_impl* f = check_file(fh);
    int rc = io_check(f, dt, count, write);
    if (rc) return rc;
    if (!write && (f->amode & MPI_MODE_SEQUENTIAL)) return GPUMPI_ERR_UNSUPPORTED_OPERATION;  // io.cu:461
    const long long got = file_xfer(f, f->pos, buf, count, dt, write);
    if (got < 0) return errno_to_mpi(got);
    f->pos += got / f->esize;
    set_status(st, got);
    return MPI_SUCCESS;
}

__device__ int io_shared(MPI_File fh, void* buf, int count, MPI_Datatype dt, MPI_Status* st, bool write) {
    MPI_File_impl* f = check_file(fh);
    int rc = io_check(f, dt, count, write);
    if (rc) return rc;
    const TypeDesc* ut = resolve_type(dt);
    const long long n = (long long)count * ut->size / f->esize;
    // the shared pointer advances by the request, in the order the atomics land (MPI-3.1 13.4.4)
    const long long pos = (long long)atomicAdd(&f->sh->shared_pos, (unsigned long long)n);
    const long long got = file_xfer(f, pos, buf, count, dt, write);
    if (got < 0) return errno_to_mpi(got);
    set_status(st, got);
    return MPI_SUCCESS;
}

// file size in bytes (host fstat)
__device__ long long file_size(MPI_File_impl* f) { return host_call(gpumpi::HIO_SIZE, f->sh->handle, 0, 0, 0); }

}  // namespace

__device__ int MPI_File_open(MPI_Comm comm, const char* filename, int amode, MPI_Info info, MPI_File* fh) {
    (void)info;
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (!fh) return GPUMPI_ERR_ARG;
    *fh = MPI_FILE_NULL;
    const int cr = comm_rank_of(c, me());
    // rank 0 checks the mode and opens; every member learns the outcome and the shared state
    long long msg[2] = {MPI_SUCCESS, 0};
    if (cr == 0) {
        int err = amode_ok(amode) ? MPI_SUCCESS : GPUMPI_ERR_AMODE;
        if (!err && !filename) err = GPUMPI_ERR_BAD_FILE;
        FileShared* sh = nullptr;
        if (!err) {
            int fl = (amode & MPI_MODE_RDONLY) ? gpumpi::HIO_F_READ
                     : (amode & MPI_MODE_WRONLY) ? gpumpi::HIO_F_WRITE
                                                 : (gpumpi::HIO_F_READ | gpumpi::HIO_F_WRITE);
            if (amode & MPI_MODE_CREATE) fl |= gpumpi::HIO_F_CREATE;
            if (amode & MPI_MODE_EXCL) fl |= gpumpi::HIO_F_EXCL;
            window_put_string(filename);
            const long long h = host_call(gpumpi::HIO_OPEN, fl, 0, 0, 0);
            if (h < 0) err = errno_to_mpi(h);
            else {
                sh = (FileShared*)malloc(sizeof(FileShared));
                if (!sh) {
                    host_call(gpumpi::HIO_CLOSE, h, 0, 0, 0);
                    err = GPUMPI_ERR_NO_MEM;
                } else {
                    sh->handle = h;
                    sh->amode = amode;
                    int k = 0;
                    for (; k < 255 && filename[k]; k++) sh->path[k] = filename[k];
                    sh->path[k] = 0;
                    // append mode: pointers start at the end of the file (default view: bytes)
                    const long long size = (amode & MPI_MODE_APPEND) ? host_call(gpumpi::HIO_SIZE, h, 0, 0, 0) : 0;
                    sh->shared_pos = size > 0 ? (unsigned long long)size : 0ULL;
                    __threadfence();
                }
            }
        }
        msg[0] = err;
        msg[1] = (long long)(size_t)sh;
    }
    int rc = MPI_Bcast(msg, 2, MPI_LONG_LONG, 0, comm);
    if (rc) return rc;
    if (msg[0] != MPI_SUCCESS) return (int)msg[0];
    FileShared* sh = (FileShared*)(size_t)msg[1];
    MPI_File_impl* f = (MPI_File_impl*)malloc(sizeof(MPI_File_impl));
    if (!f) return GPUMPI_ERR_NO_MEM;
    memset(f, 0, sizeof(MPI_File_impl));
    f->magic = FILE_MAGIC;
    f->sh = sh;
    f->comm = comm;
    f->amode = amode;
    f->disp = 0;
    f->etype = MPI_CHAR;  // the initial view: the reference's choice (io.cu:222), one byte like MPI_BYTE
    f->filetype = MPI_CHAR;
    f->esize = 1;
    f->ft = *resolve_type(MPI_CHAR);
    f->pos = (long long)*(volatile unsigned long long*)&sh->shared_pos;  // 0, or the end (append mode)
    const char nat[] = "native";
    for (int k = 0; k < 7; k++) f->datarep[k] = nat[k];
    *fh = f;
    return MPI_SUCCESS;
}

__device__ int MPI_File_close(MPI_File* fh) {
    if (!fh) return GPUMPI_ERR_ARG;
    MPI_File_impl* f = check_file(*fh);
    if (!f) return GPUMPI_ERR_FILE;
    int rc = MPI_Barrier(f->comm);  // every member's accesses are done
    if (rc) return rc;
    MPI_Comm_impl* c = check_comm(f->comm);
    if (c && comm_rank_of(c, me()) == 0) {
        FileShared* sh = f->sh;
        const long long e = host_call(gpumpi::HIO_CLOSE, sh->handle, 0, 0, 0);
        if (e < 0) rc = errno_to_mpi(e);
        if (sh->amode & MPI_MODE_DELETE_ON_CLOSE) {
            window_put_string(sh->path);
            host_call(gpumpi::HIO_REMOVE, 0, 0, 0, 0);
        }
        free(sh);
    }
    f->magic = 0;
    free(f);
    *fh = MPI_FILE_NULL;
    return rc;
}

__device__ int MPI_File_delete(const char* filename, MPI_Info info) {
    (void)info;
    if (!window_put_string(filename)) return GPUMPI_ERR_BAD_FILE;
    const long long e = host_call(gpumpi::HIO_REMOVE, 0, 0, 0, 0);
    return e < 0 ? errno_to_mpi(e) : MPI_SUCCESS;
}

__device__ int MPI_File_get_size(MPI_File fh, MPI_Offset* size) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    if (!size) return GPUMPI_ERR_ARG;
    const long long s = file_size(f);
    if (s < 0) return errno_to_mpi(s);
    *size = s;
    return MPI_SUCCESS;
}

__device__ int MPI_File_set_size(MPI_File fh, MPI_Offset size) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    if (size < 0) return GPUMPI_ERR_ARG;
    if (f->amode & MPI_MODE_RDONLY) return GPUMPI_ERR_READ_ONLY;
    int rc = MPI_Barrier(f->comm);
    if (rc) return rc;
    MPI_Comm_impl* c = check_comm(f->comm);
    long long e = 0;
    if (c && comm_rank_of(c, me()) == 0) e = host_call(gpumpi::HIO_TRUNCATE, f->sh->handle, size, 0, 0);
    rc = MPI_Bcast(&e, 1, MPI_LONG_LONG, 0, f->comm);
    if (rc) return rc;
    return e < 0 ? errno_to_mpi(e) : MPI_SUCCESS;
}

__device__ int MPI_File_sync(MPI_File fh) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    int rc = MPI_Barrier(f->comm);
    if (rc) return rc;
    MPI_Comm_impl* c = check_comm(f->comm);
    long long e = 0;
    if (c && comm_rank_of(c, me()) == 0) e = host_call(gpumpi::HIO_FLUSH, f->sh->handle, 0, 0, 0);
    rc = MPI_Bcast(&e, 1, MPI_LONG_LONG, 0, f->comm);
    if (rc) return rc;
    return e < 0 ? errno_to_mpi(e) : MPI_SUCCESS;
}

__device__ int MPI_File_get_amode(MPI_File fh, int* amode) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    if (!amode) return GPUMPI_ERR_ARG;
    *amode = f->amode;
    return MPI_SUCCESS;
}

__device__ int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype,
                                 const char* datarep, MPI_Info info) {
    (void)info;
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    const TypeDesc* et = resolve_type(etype);
    const TypeDesc* ft = resolve_type(filetype);
    if (!et || !ft || et->size <= 0 || ft->size <= 0 || ft->size % et->size) return GPUMPI_ERR_TYPE;
    const char nat[] = "native";
    if (datarep) {
        for (int k = 0; k < 7; k++)
            if (datarep[k] != nat[k]) return GPUMPI_ERR_UNSUPPORTED_DATAREP;
    }
    if (disp == MPI_DISPLACEMENT_CURRENT) {
        if (!(f->amode & MPI_MODE_SEQUENTIAL)) return GPUMPI_ERR_ARG;
        disp = f->disp + desc_map(&f->ft, f->pos * f->esize);
    }
    if (disp < 0) return GPUMPI_ERR_ARG;
    f->disp = disp;
    f->etype = etype;
    f->filetype = filetype;
    f->esize = et->size;
    f->ft = *ft;
    for (int k = 0; k < 7; k++) f->datarep[k] = nat[k];
    f->pos = 0;
    // collective: the shared pointer restarts at zero once every member has set its view
    int rc = MPI_Barrier(f->comm);
    if (rc) return rc;
    MPI_Comm_impl* c = check_comm(f->comm);
    if (c && comm_rank_of(c, me()) == 0) atomicExch(&f->sh->shared_pos, 0ULL);
    return MPI_Barrier(f->comm);
}

__device__ int MPI_File_get_view(MPI_File fh, MPI_Offset* disp, MPI_Datatype* etype, MPI_Datatype* filetype,
                                 char* datarep) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    if (disp) *disp = f->disp;
    if (etype) *etype = (MPI_Datatype)f->etype;
    if (filetype) *filetype = (MPI_Datatype)f->filetype;
    if (datarep)
        for (int k = 0; k < 16; k++) {
            datarep[k] = f->datarep[k];
            if (!f->datarep[k]) break;
        }
    return MPI_SUCCESS;
}

__device__ int MPI_File_read(MPI_File fh, void* buf, int count, MPI_Datatype dt, MPI_Status* st) {
    return io_ind(fh, buf, count, dt, st, false);
}
__device__ int MPI_File_write(MPI_File fh, const void* buf, int count, MPI_Datatype dt, MPI_Status* st) {
    return io_ind(fh, (void*)buf, count, dt, st, true);
}
__device__ int MPI_File_read_at(MPI_File fh, MPI_Offset offset, void* buf, int count, MPI_Datatype dt,
                                MPI_Status* st) {
    return io_at(fh, offset, buf, count, dt, st, false);
}
__device__ int MPI_File_write_at(MPI_File fh, MPI_Offset offset, const void* buf, int count, MPI_Datatype dt,
                                 MPI_Status* st) {
    return io_at(fh, offset, (void*)buf, count, dt, st, true);
}
// collective forms: every member calls; each moves its own data (no ordering beyond the independent forms)
__device__ int MPI_File_read_all(MPI_File fh, void* buf, int count, MPI_Datatype dt, MPI_Status* st) {
    return io_ind(fh, buf, count, dt, st, false);
}
__device__ int MPI_File_write_all(MPI_File fh, const void* buf, int count, MPI_Datatype dt, MPI_Status* st) {
    return io_ind(fh, (void*)buf, count, dt, st, true);
}
__device__ int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void* buf, int count, MPI_Datatype dt,
                                    MPI_Status* st) {
    return io_at(fh, offset, buf, count, dt, st, false);
}
__device__ int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void* buf, int count, MPI_Datatype dt,
                                     MPI_Status* st) {
    return io_at(fh, offset, (void*)buf, count, dt, st, true);
}
__device__ int MPI_File_read_shared(MPI_File fh, void* buf, int count, MPI_Datatype dt, MPI_Status* st) {
    return io_shared(fh, buf, count, dt, st, false);
}
__device__ int MPI_File_write_shared(MPI_File fh, const void* buf, int count, MPI_Datatype dt, MPI_Status* st) {
    return io_shared(fh, (void*)buf, count, dt, st, true);
}

__device__ int MPI_File_seek(MPI_File fh, MPI_Offset offset, int whence) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    if (f->amode & MPI_MODE_SEQUENTIAL) return GPUMPI_ERR_UNSUPPORTED_OPERATION;
    long long p;
    if (whence == MPI_SEEK_SET) {
        p = offset;
    } else if (whence == MPI_SEEK_CUR) {
        p = f->pos + offset;
    } else if (whence == MPI_SEEK_END) {
        // the end of the file in etypes of the view (a view whose filetype is contiguous)
        if (!desc_contiguous(&f->ft) && !(f->ft.nlev == 0 && f->ft.size == f->ft.extent))
            return GPUMPI_ERR_UNSUPPORTED_OPERATION;
        const long long s = file_size(f);
        if (s < 0) return errno_to_mpi(s);
        const long long past = s - f->disp;
        p = (past > 0 ? (past + f->esize - 1) / f->esize : 0) + offset;
    } else {
        return GPUMPI_ERR_ARG;
    }
    if (p < 0) return GPUMPI_ERR_ARG;
    f->pos = p;
    return MPI_SUCCESS;
}

__device__ int MPI_File_get_position(MPI_File fh, MPI_Offset* offset) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    if (!offset) return GPUMPI_ERR_ARG;
    *offset = f->pos;
    return MPI_SUCCESS;
}

__device__ int MPI_File_seek_shared(MPI_File fh, MPI_Offset offset, int whence) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    if (whence != MPI_SEEK_SET && whence != MPI_SEEK_CUR && whence != MPI_SEEK_END) return GPUMPI_ERR_ARG;
    int rc = MPI_Barrier(f->comm);  // collective: every member's earlier shared accesses have landed
    if (rc) return rc;
    MPI_Comm_impl* c = check_comm(f->comm);
    long long err = MPI_SUCCESS;
    if (c && comm_rank_of(c, me()) == 0) {
        long long p = offset;
        if (whence == MPI_SEEK_CUR) p += (long long)*(volatile unsigned long long*)&f->sh->shared_pos;
        if (whence == MPI_SEEK_END) {
            const long long s = file_size(f);
            p += s > f->disp ? (s - f->disp + f->esize - 1) / f->esize : 0;
        }
        if (p < 0) err = GPUMPI_ERR_ARG;
        else atomicExch(&f->sh->shared_pos, (unsigned long long)p);
    }
    rc = MPI_Bcast(&err, 1, MPI_LONG_LONG, 0, f->comm);
    return rc ? rc : (int)err;
}

__device__ int MPI_File_get_position_shared(MPI_File fh, MPI_Offset* offset) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    if (!offset) return GPUMPI_ERR_ARG;
    *offset = (long long)*(volatile unsigned long long*)&f->sh->shared_pos;
    return MPI_SUCCESS;
}

__device__ int MPI_File_get_byte_offset(MPI_File fh, MPI_Offset offset, MPI_Offset* disp) {
    MPI_File_impl* f = check_file(fh);
    if (!f) return GPUMPI_ERR_FILE;
    if (!disp || offset < 0) return GPUMPI_ERR_ARG;
    *disp = f->disp + desc_map(&f->ft, offset * f->esize);
    return MPI_SUCCESS;
}
