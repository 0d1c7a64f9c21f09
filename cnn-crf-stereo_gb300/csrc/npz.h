// npz.h -- reader and writer of numpy .npz archives of float32 arrays (the
// parameter format the reference reads with cnpy::npz_load,
// stereo/operators/operator.cpp:55-85; the writer saves training checkpoints
// in the same layout).
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

// One float32 array of an archive to write: `key` (".npy" appended), C-order
// data of the given shape (an empty shape is a 0-d scalar).
struct NpzMember {
    std::string key;
    const float *data;
    std::vector<int64_t> shape;
};

// Write an uncompressed (STORED) .npz that numpy.load and npz_load read:
// one .npy (format 1.0, '<f4', C order) per member.  The archive is written
// to `path`.tmp and renamed over `path`, so a failed write leaves any older
// file in place.  EIO when the file cannot be written, EUNSUPPORTED above
// the plain zip format's 4 GiB / 65535-member limits.
int npz_save(const std::string &path, const std::vector<NpzMember> &members);

// Raw DEFLATE (RFC 1951) decoder: inflate `in` into exactly `out_size` bytes.
bool inflate_raw(const uint8_t *in, size_t in_size, std::vector<uint8_t> *out, size_t out_size);

} // namespace cnncrf
