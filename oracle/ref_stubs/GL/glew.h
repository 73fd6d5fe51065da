/*
 * Minimal stand-in for <GL/glew.h>, used only to compile the reference's
 * CPU shadow-build sources (CompressedShadow.cpp, CompressedShadowUtil.cpp,
 * MinMaxHierarchy.cpp) as a test oracle.  Those files include GL headers
 * through cpvs.h / Texture.h but never call GL on the build or lookup path;
 * the inline texture helpers in Texture.h only need the names below to exist.
 * Every function is a no-op.  Test infrastructure only.
 */
#ifndef ORACLE_STUB_GLEW_H
#define ORACLE_STUB_GLEW_H

typedef unsigned int GLenum;
typedef unsigned int GLuint;
typedef int GLint;
typedef int GLsizei;
typedef unsigned char GLboolean;
typedef float GLfloat;

#define GL_FALSE 0
#define GL_TRUE 1
#define GL_NO_ERROR 0
#define GL_TEXTURE0 0x84C0
#define GL_TEXTURE_1D 0x0DE0
#define GL_TEXTURE_2D 0x0DE1
#define GL_DEPTH_COMPONENT 0x1902

static inline void glGenTextures(GLsizei, GLuint* ids) { if (ids) *ids = 0; }
static inline void glDeleteTextures(GLsizei, const GLuint*) {}
static inline void glActiveTexture(GLenum) {}
static inline void glBindTexture(GLenum, GLuint) {}
static inline void glBindImageTexture(GLuint, GLuint, GLint, GLboolean, GLint, GLenum, GLenum) {}
static inline GLenum glGetError(void) { return GL_NO_ERROR; }

#endif
