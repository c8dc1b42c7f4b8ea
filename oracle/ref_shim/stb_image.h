/* Stand-in for the image-decoding header the reference's core/image.cc includes.
 * The oracle build never reads image files (scenes are procedural), so every
 * entry point reports failure.  Written for this project; declares only the
 * names core/image.cc uses. Oracle-only test infrastructure. */
#ifndef SPICA_ORACLE_STB_IMAGE_STUB_H
#define SPICA_ORACLE_STB_IMAGE_STUB_H
#include <stdint.h>
enum { STBI_default = 0, STBI_grey = 1, STBI_grey_alpha = 2, STBI_rgb = 3, STBI_rgb_alpha = 4 };
static inline unsigned char *stbi_load(const char *, int *w, int *h, int *c, int) {
    if (w) *w = 0;
    if (h) *h = 0;
    if (c) *c = 0;
    return 0;
}
static inline void stbi_image_free(void *) {}
#endif
