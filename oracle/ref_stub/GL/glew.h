/* Stand-in for <GL/glew.h> when the reference's octree.c is compiled for the
 * oracle: octree.c includes it only for the GL scalar typedefs. */
#ifndef QB_REF_STUB_GLEW_H
#define QB_REF_STUB_GLEW_H
typedef int          GLint;
typedef unsigned int GLuint;
typedef float        GLfloat;
#endif
