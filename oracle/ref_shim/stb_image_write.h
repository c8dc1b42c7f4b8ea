/* Stand-in for the image-encoding header the reference's core/image.cc includes.
 * Image output is out of scope for the oracle, so writes report failure (0).
 * Written for this project. Oracle-only test infrastructure. */
#ifndef SPICA_ORACLE_STB_IMAGE_WRITE_STUB_H
#define SPICA_ORACLE_STB_IMAGE_WRITE_STUB_H
static inline int stbi_write_bmp(const char *, int, int, int, const void *) { return 0; }
static inline int stbi_write_png(const char *, int, int, int, const void *, int) { return 0; }
#endif
