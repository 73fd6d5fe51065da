/* Empty stand-in for <GLFW/glfw3.h>: the reference's shadow-build sources
 * include it but use nothing from it.  Test infrastructure only. */
#ifndef ORACLE_STUB_GLFW3_H
#define ORACLE_STUB_GLFW3_H
#endif
