// gpumpi_stdio.h.cuh — file and stream output from ranks, performed by the host process.
//
// Requests travel over the world's device -> host channel (a ring in page-locked host memory served by
// a host thread of the world); each call waits for the host's answer, bounded by the world's timeout.
// The reference's device libc has no working file access (gpu_libs/gpu_libc/stdio.cu:32-66: fopen
// returns nullptr, fclose/fputs/puts trap) and prints through CUDA's device printf, which appears only
// when the kernel ends.  gpumpi_printf / gpumpi_fprintf format with the host's printf and reach the
// stream in call order, interleaved correctly with the host process's own output.
//
// Call from thread 0 of a rank block, like every MPI function.  A converted program that defines
// GPUMPI_STDIO_NAMES before including this header gets the standard names (FILE, fopen, fprintf, ...)
// mapped onto these functions.
#pragma once
#include <stdarg.h>
#include <stddef.h>

struct gpumpi_FILE_impl;
typedef struct gpumpi_FILE_impl gpumpi_FILE;
#define gpumpi_stdout ((gpumpi_FILE*)1)
#define gpumpi_stderr ((gpumpi_FILE*)2)

// mode: "r", "r+", "w", "w+", "a", "a+" (a "b" is accepted and ignored; "x" adds exclusive creation)
__device__ gpumpi_FILE* gpumpi_fopen(const char* path, const char* mode);
__device__ int gpumpi_fclose(gpumpi_FILE* f);
__device__ size_t gpumpi_fwrite(const void* ptr, size_t size, size_t nmemb, gpumpi_FILE* f);
__device__ size_t gpumpi_fread(void* ptr, size_t size, size_t nmemb, gpumpi_FILE* f);
__device__ int gpumpi_fputs(const char* s, gpumpi_FILE* f);
__device__ int gpumpi_puts(const char* s);
__device__ int gpumpi_fflush(gpumpi_FILE* f);
__device__ int gpumpi_remove(const char* path);
// Conversions: d i u x X o c s f F e E g G a A p with flags, width, precision ('*' too) and length
// modifiers; the values are read on the device and formatted by the host.
__device__ int gpumpi_fprintf(gpumpi_FILE* f, const char* fmt, ...);
__device__ int gpumpi_printf(const char* fmt, ...);
// Formatted into dst by the host (the same conversions); the text is cut to the rank's host-channel window
// (host_window_bytes - 1 characters) and to size - 1 for the n forms; returns the full length, -1 on error.
__device__ int gpumpi_sprintf(char* dst, const char* fmt, ...);
__device__ int gpumpi_snprintf(char* dst, size_t size, const char* fmt, ...);
__device__ int gpumpi_vsprintf(char* dst, const char* fmt, va_list ap);
__device__ int gpumpi_vsnprintf(char* dst, size_t size, const char* fmt, va_list ap);

#ifdef GPUMPI_STDIO_NAMES
#define FILE gpumpi_FILE
#undef stdout
#undef stderr
#define stdout gpumpi_stdout
#define stderr gpumpi_stderr
#define fopen gpumpi_fopen
#define fclose gpumpi_fclose
#define fwrite gpumpi_fwrite
#define fread gpumpi_fread
#define fputs gpumpi_fputs
#define puts gpumpi_puts
#define fflush gpumpi_fflush
#define remove gpumpi_remove
#define fprintf gpumpi_fprintf
#undef printf
#define printf gpumpi_printf
#define sprintf gpumpi_sprintf
#define snprintf gpumpi_snprintf
#define vsprintf gpumpi_vsprintf
#define vsnprintf gpumpi_vsnprintf
#endif
