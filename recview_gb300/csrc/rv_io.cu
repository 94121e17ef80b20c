// Output side of a reconstruction (host code): the 16-bit TIFF RecView writes for each slice
// (WriteTifMonochrome16, source/general.cpp:1313-1470), its ImageDescription fields
// (source/gazoDoc.cpp:1985-1988) and the physical scale of the rescaled values
// (source/gazoDoc.cpp:3998-4006).  Files are byte-identical to RecView's.
#include <limits.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "rv_internal.h"

namespace {

// little-endian writers with the reference's field widths (an LLP64 build: long = 32 bits)
void put16(std::vector<unsigned char>& b, uint16_t v) {
    b.push_back((unsigned char)(v & 0xff));
    b.push_back((unsigned char)(v >> 8));
}
void put32(std::vector<unsigned char>& b, uint32_t v) {
    for (int i = 0; i < 4; i++) b.push_back((unsigned char)((v >> (8 * i)) & 0xff));
}
void entry(std::vector<unsigned char>& b, uint16_t tag, uint16_t type, uint32_t count, uint32_t value) {
    put16(b, tag);
    put16(b, type);
    put32(b, count);
    put32(b, value);
}
// the reference pads short strings with four blanks, cuts long ones to 199 characters and counts
// the terminating NUL (source/general.cpp:1363-1368,1376-1381)
std::string tif_string(const char* s, uint32_t* n) {
    std::string t = s ? s : "";
    if (t.size() < 4) t += "    ";
    if (t.size() > 199) t = t.substr(0, 199);
    *n = (uint32_t)t.size() + 1;
    return t;
}

}  // namespace

using namespace rv;

extern "C" long long RvTiff16Bytes(const int* slice, int height, int width, const char* description,
                                   const char* artist, unsigned char* out, long long cap) {
    if (!slice || height < 1 || width < 1) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvTiff16Bytes: invalid argument");
        return -RV_ERR_BAD_ARGUMENT;
    }
    std::vector<unsigned char> b;
    const uint32_t offset = 8;
    uint32_t oDirEnt = offset + (uint32_t)height * (uint32_t)width * 2u;
    b.push_back('I');
    b.push_back('I');
    put16(b, 42);
    put32(b, oDirEnt);
    for (long long i = 0; i < (long long)height * width; i++) {
        const int v = slice[i];
        put16(b, v > 0 ? (uint16_t)v : (uint16_t)0);
    }
    const uint16_t nDir = 12;
    put16(b, nDir);
    uint32_t nDesc = 0, nArtist = 0;
    const std::string desc = tif_string(description, &nDesc);
    const std::string art = tif_string(artist ? artist : "SP-uCT, gazoView", &nArtist);
    const uint32_t oDesc = oDirEnt + 2 + nDir * 12 + 4;
    uint32_t oStripOffsets = oDesc + nDesc;
    if (nDesc & 1) oStripOffsets++;
    const uint32_t oStripByteCounts = oStripOffsets + (uint32_t)height * 4;
    const uint32_t oArtist = oStripByteCounts + (uint32_t)height * 4;
    // tag numbers and types: source/constants.h:11-35
    entry(b, 0x0100, 3, 1, (uint32_t)width);
    entry(b, 0x0101, 3, 1, (uint32_t)height);
    entry(b, 0x0102, 3, 1, 16);
    entry(b, 0x0103, 3, 1, 1);
    entry(b, 0x0106, 3, 1, 1);
    entry(b, 0x010e, 2, nDesc, oDesc);
    entry(b, 0x0111, 4, (uint32_t)height, oStripOffsets);
    entry(b, 0x0115, 3, 1, 1);
    entry(b, 0x0116, 3, 1, 1);
    entry(b, 0x0117, 4, (uint32_t)height, oStripByteCounts);
    entry(b, 0x011c, 3, 1, 1);
    entry(b, 0x013b, 2, nArtist, oArtist);
    put32(b, 0);
    b.insert(b.end(), desc.begin(), desc.end());
    b.push_back(0);
    if (nDesc & 1) b.push_back(0);
    for (int i = 0; i < height; i++) put32(b, offset + (uint32_t)i * (uint32_t)width * 2u);
    for (int i = 0; i < height; i++) put32(b, (uint32_t)width * 2u);
    b.insert(b.end(), art.begin(), art.end());
    b.push_back(0);
    if (nArtist & 1) b.push_back(0);
    if (out && (long long)b.size() <= cap) memcpy(out, b.data(), b.size());
    return (long long)b.size();
}

extern "C" int RvWriteTiff16(const char* path, const int* slice, int height, int width, const char* description,
                             const char* artist) {
    if (!path) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvWriteTiff16: NULL path");
        return RV_ERR_BAD_ARGUMENT;
    }
    const long long n = RvTiff16Bytes(slice, height, width, description, artist, nullptr, 0);
    if (n < 0) return (int)-n;
    std::vector<unsigned char> b((size_t)n);
    RvTiff16Bytes(slice, height, width, description, artist, b.data(), n);
    FILE* f = fopen(path, "wb");
    if (!f) {
        set_error(RV_ERR_UNSUPPORTED, std::string("RvWriteTiff16: cannot open ") + path);
        return RV_ERR_UNSUPPORTED;
    }
    const size_t w = fwrite(b.data(), 1, b.size(), f);
    fclose(f);
    if (w != b.size()) {
        set_error(RV_ERR_UNSUPPORTED, std::string("RvWriteTiff16: short write to ") + path);
        return RV_ERR_UNSUPPORTED;
    }
    return 0;
}

extern "C" int RvPixelScale(int nSinogr, double pixelWidth, int iBinning, int ipintp, int imin, int imax, int zernike,
                            float* pixelBase, float* pixelDiv) {
    // source/gazoDoc.cpp:3997-4006
    if (!pixelBase || !pixelDiv || nSinogr < 1 || ipintp < 1 || iBinning < 1) return RV_ERR_BAD_ARGUMENT;
    if (imin == imax) imax++;
    const double scaleFactor = 6.2831853 * 10000. / (pixelWidth * iBinning);
    double sc = scaleFactor / (RV_LOG_SCALE * RV_BACKPROJ_SCALE * nSinogr);
    if (zernike) sc = scaleFactor / (1000 * RV_BACKPROJ_SCALE * nSinogr);
    *pixelBase = (float)(sc * ipintp * imin);
    *pixelDiv = (float)((USHRT_MAX - 1) / sc / (imax - imin) / ipintp);
    return 0;
}

extern "C" int RvImageDescription(char* out, int cap, int nSinogr, double pixelWidth, float pixelDiv, float pixelBase,
                                  double centre, int filterKind) {
    // the fields CGazoDoc::BatchReconst stores in each slice's TIFF (source/gazoDoc.cpp:1985-1988)
    if (!out || cap < 1) return RV_ERR_BAD_ARGUMENT;
    const int n = snprintf(out, (size_t)cap, "%d\t%.6f\t%.6f\t%.6f\t%.6f\t%d\t%.6f\t%.6f ", nSinogr, pixelWidth,
                           (double)pixelDiv, (double)pixelBase, centre, filterKind + 1, 55.111697, 0.461227);
    return (n >= 0 && n < cap) ? 0 : RV_ERR_BAD_ARGUMENT;
}
