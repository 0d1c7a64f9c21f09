// npz.h -- reader for numpy .npz archives of float32 arrays (the checkpoint
// format the reference reads with cnpy::npz_load, stereo/operators/operator.cpp:55-85).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace cnncrf {

struct NpyArray {
    std::vector<int64_t> shape;
    std::vector<float> data; // C order
};

// Load member `key` (".npy" appended) of the archive.  Returns a cnncrf_status;
// EIO for a missing / corrupt file or member, ESHAPE for a non-float32 or
// Fortran-ordered array.  Supports STORED and DEFLATE members and ZIP64 sizes.
int npz_load(const std::string &path, const std::string &key, NpyArray *out);

// Raw DEFLATE (RFC 1951) decoder: inflate `in` into exactly `out_size` bytes.
bool inflate_raw(const uint8_t *in, size_t in_size, std::vector<uint8_t> *out, size_t out_size);

} // namespace cnncrf
