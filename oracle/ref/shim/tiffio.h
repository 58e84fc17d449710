/* Stand-in for the libtiff header, for compiling the reference's own sources
 * into the oracle's reference build (test infrastructure only).  The
 * reference functions that build calls write no TIFF files; the TIFF
 * functions of the same source files are compiled against these
 * declarations and abort if called.  Tag values are those of the TIFF 6.0
 * specification. */
#ifndef TDM_REF_TIFFIO_SHIM_H
#define TDM_REF_TIFFIO_SHIM_H
#include <stdint.h>
#include <stdlib.h>

typedef struct tdm_ref_tiff_s TIFF;
typedef uint8_t uint8;
typedef uint16_t uint16;
typedef uint32_t uint32;
typedef int16_t int16;
typedef int32_t int32;
typedef uint32_t ttag_t;
typedef int64_t tmsize_t;
typedef void* tdata_t;
typedef uint32_t tstrip_t;
typedef int64_t tsize_t;

#define TIFFTAG_SUBFILETYPE 254
#define FILETYPE_PAGE 0x2
#define TIFFTAG_IMAGEWIDTH 256
#define TIFFTAG_IMAGELENGTH 257
#define TIFFTAG_BITSPERSAMPLE 258
#define TIFFTAG_COMPRESSION 259
#define COMPRESSION_NONE 1
#define COMPRESSION_LZW 5
#define COMPRESSION_DEFLATE 32946
#define TIFFTAG_PHOTOMETRIC 262
#define PHOTOMETRIC_MINISBLACK 1
#define TIFFTAG_ORIENTATION 274
#define ORIENTATION_TOPLEFT 1
#define ORIENTATION_BOTLEFT 4
#define TIFFTAG_SAMPLESPERPIXEL 277
#define TIFFTAG_ROWSPERSTRIP 278
#define TIFFTAG_XRESOLUTION 282
#define TIFFTAG_YRESOLUTION 283
#define TIFFTAG_PLANARCONFIG 284
#define PLANARCONFIG_CONTIG 1
#define TIFFTAG_RESOLUTIONUNIT 296
#define RESUNIT_CENTIMETER 3
#define TIFFTAG_PAGENUMBER 297
#define TIFFTAG_SAMPLEFORMAT 339
#define SAMPLEFORMAT_IEEEFP 3

#ifdef __cplusplus
extern "C" {
#endif
static inline TIFF* TIFFOpen(const char*, const char*) { abort(); }
static inline void TIFFClose(TIFF*) { abort(); }
static inline int TIFFSetField(TIFF*, uint32_t, ...) { abort(); }
static inline int TIFFGetField(TIFF*, uint32_t, ...) { abort(); }
static inline int TIFFWriteDirectory(TIFF*) { abort(); }
static inline int TIFFWriteScanline(TIFF*, void*, uint32_t, uint16_t) { abort(); }
static inline int TIFFReadScanline(TIFF*, void*, uint32_t, uint16_t) { abort(); }
static inline tmsize_t TIFFWriteEncodedStrip(TIFF*, uint32_t, void*, tmsize_t) { abort(); }
static inline tmsize_t TIFFStripSize(TIFF*) { abort(); }
static inline uint32_t TIFFNumberOfStrips(TIFF*) { abort(); }
static inline void* _TIFFmalloc(tmsize_t) { abort(); }
static inline void _TIFFfree(void*) { abort(); }
#ifdef __cplusplus
}
#endif
#define TIFFmalloc _TIFFmalloc
#define TIFFfree _TIFFfree
#endif
