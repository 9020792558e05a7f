/* stub: GL type names only, so that the compute sources compile headless */
typedef unsigned int GLuint; typedef int GLint; typedef unsigned int GLenum; typedef int GLsizei;
