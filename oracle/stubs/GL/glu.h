/* Empty: the reference includes <GL/glu.h> but its headless numerical code uses nothing from it. */
