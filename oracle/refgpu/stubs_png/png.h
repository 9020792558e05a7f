/* stub: declarations only, so that the reference's image export (texture_save.cu) parses when
 * its device code is compiled into a cubin; no libpng function is ever called. */
#ifndef REFGPU_STUB_PNG_H
#define REFGPU_STUB_PNG_H
#include <csetjmp>
#include <cstdio>

typedef struct png_struct_def *png_structp;
typedef struct png_info_def *png_infop;
typedef unsigned char *png_bytep;
typedef png_structp *png_structpp;
typedef png_infop *png_infopp;

#define PNG_LIBPNG_VER_STRING "stub"
#define PNG_COLOR_TYPE_GRAY 0
#define PNG_COLOR_TYPE_RGB 2
#define PNG_INTERLACE_NONE 0
#define PNG_COMPRESSION_TYPE_DEFAULT 0
#define PNG_FILTER_TYPE_DEFAULT 0
#define PNG_sRGB_INTENT_PERCEPTUAL 0

png_structp png_create_write_struct(const char *, void *, void *, void *);
png_infop png_create_info_struct(png_structp);
void png_destroy_write_struct(png_structpp, png_infopp);
std::jmp_buf &png_jmpbuf_ref(png_structp);
#define png_jmpbuf(p) (png_jmpbuf_ref(p))
void png_init_io(png_structp, FILE *);
void png_set_IHDR(png_structp, png_infop, unsigned, unsigned, int, int, int, int, int);
void png_set_sRGB(png_structp, png_infop, int);
void png_write_info(png_structp, png_infop);
void png_set_swap(png_structp);
void png_write_image(png_structp, png_bytep *);
void png_write_end(png_structp, png_infop);
int fopen_s(FILE **, const char *, const char *);
#endif
