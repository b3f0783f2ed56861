/* Headless stand-in for GLEW, used only to compile the reference's MPM core
 * as a CPU oracle.  The reference's Mesh constructor (mesh.hpp:28-37) calls
 * three buffer functions; here they do nothing.  No GL context ever exists. */
#pragma once
#include <cstddef>
typedef unsigned int GLuint;
typedef unsigned int GLenum;
typedef float GLfloat;
typedef unsigned char GLubyte;
typedef std::ptrdiff_t GLsizeiptr;
#define GL_ARRAY_BUFFER 0x8892
#define GL_STATIC_DRAW 0x88E4
inline void glGenBuffers(int, GLuint* b) { if (b) *b = 0; }
inline void glBindBuffer(GLenum, GLuint) {}
inline void glBufferData(GLenum, GLsizeiptr, const void*, GLenum) {}
