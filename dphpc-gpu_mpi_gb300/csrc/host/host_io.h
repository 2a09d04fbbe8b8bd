// host_io.h — creation and teardown of a world's device -> host request channel (host_io.cu).
#pragma once
#include <cstddef>
#include <string>

namespace gpumpi {
struct HostIO;
}
struct HostService;

// Allocates the mapped ring, response slots and payload windows (window_bytes per rank), fills the
// device-side descriptor `desc` (d_tail and d_broken are device memory the caller owns, zeroed), and starts
// the service thread.  Returns nullptr (and a reason in *err) when an allocation fails.
HostService* hio_create(int nranks, size_t window_bytes, unsigned long long* d_tail, unsigned* d_broken,
                        gpumpi::HostIO* desc, std::string* err);
// Stops the service thread, closes the files the ranks left open and frees the mapped memory.
void hio_destroy(HostService* s);
