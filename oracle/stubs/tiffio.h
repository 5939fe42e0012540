/* No-op stand-ins for the libtiff calls of the reference's frame writer (project-written). */
#ifndef WO_STUB_TIFFIO_H
#define WO_STUB_TIFFIO_H
#include <stdint.h>
typedef struct TIFF TIFF;
enum { TIFFTAG_SAMPLESPERPIXEL, TIFFTAG_ROWSPERSTRIP, TIFFTAG_PLANARCONFIG, TIFFTAG_PHOTOMETRIC,
       TIFFTAG_ORIENTATION, TIFFTAG_IMAGEWIDTH, TIFFTAG_IMAGELENGTH, TIFFTAG_IMAGEDESCRIPTION,
       TIFFTAG_COMPRESSION, TIFFTAG_BITSPERSAMPLE, PLANARCONFIG_CONTIG, PHOTOMETRIC_RGB,
       ORIENTATION_BOTLEFT, COMPRESSION_LZW };
static inline TIFF *TIFFOpen(const char *a, const char *b) { (void)a; (void)b; return 0; }
static inline int TIFFSetField(TIFF *t, int tag, ...) { (void)t; (void)tag; return 0; }
static inline int TIFFWriteScanline(TIFF *t, void *p, int r, int s) { (void)t; (void)p; (void)r; (void)s; return 0; }
static inline void TIFFClose(TIFF *t) { (void)t; }
#endif
