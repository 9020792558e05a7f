/* stub: declarations only (image loading is off the compute path) */
extern "C" unsigned char *stbi_load(const char *, int *, int *, int *, int);
extern "C" void stbi_image_free(void *);
