/* No-op stand-ins for the GLUT/GL entry points the reference's headless build
 * references.  Project-written: declarations with empty bodies, so that the
 * reference's numerical code compiles without any graphics library.  No GL code
 * path is executed by the oracle drivers. */
#ifndef WO_STUB_GLUT_H
#define WO_STUB_GLUT_H
#include <stdio.h>
#include <stdlib.h>
typedef unsigned char GLubyte;
enum { GL_LINE_LOOP, GL_LINE_STRIP, GL_LINES, GL_QUADS, GL_LINE_SMOOTH, GL_TRIANGLE_FAN,
       GL_COLOR_BUFFER_BIT, GL_UNSIGNED_BYTE, GL_SCISSOR_TEST, GL_RGB, GL_PACK_ALIGNMENT,
       GLUT_RGB, GLUT_DOUBLE, GLUT_DEPTH };
#define GLUT_BITMAP_TIMES_ROMAN_24 0
#define GLUT_BITMAP_8_BY_13 0
#define GLUT_BITMAP_9_BY_15 0
static inline void glBegin(int m) { (void)m; }
static inline void glEnd(void) {}
static inline void glClear(int m) { (void)m; }
static inline void glClearColor(double a, double b, double c, double d) { (void)a; (void)b; (void)c; (void)d; }
static inline void glColor3f(double a, double b, double c) { (void)a; (void)b; (void)c; }
static inline void glDisable(int x) { (void)x; }
static inline void glEnable(int x) { (void)x; }
static inline void glLineWidth(double w) { (void)w; }
static inline void glOrtho(double a, double b, double c, double d, double e, double f) { (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; }
static inline void glPixelStorei(int a, int b) { (void)a; (void)b; }
static inline void glPopMatrix(void) {}
static inline void glPushMatrix(void) {}
static inline void glRasterPos2d(double x, double y) { (void)x; (void)y; }
static inline void glReadPixels(int x, int y, int w, int h, int f, int t, void *p) { (void)x; (void)y; (void)w; (void)h; (void)f; (void)t; (void)p; }
static inline void glScissor(double a, double b, double c, double d) { (void)a; (void)b; (void)c; (void)d; }
static inline void glVertex2d(double a, double b) { (void)a; (void)b; }
static inline void glVertex2i(int a, int b) { (void)a; (void)b; }
static inline void glutBitmapCharacter(int f, int c) { (void)f; (void)c; }
static inline int glutCreateWindow(const char *s) { (void)s; return 0; }
static inline void glutDestroyWindow(int w) { (void)w; }
static inline void glutDisplayFunc(void (*f)(void)) { (void)f; }
static inline int glutGetWindow(void) { return 0; }
static inline void glutInit(int *a, char **b) { (void)a; (void)b; }
static inline void glutInitDisplayMode(int m) { (void)m; }
static inline void glutInitWindowSize(int w, int h) { (void)w; (void)h; }
static inline void glutMainLoop(void) {}
static inline void glutSwapBuffers(void) {}
#endif
