/* Empty stand-in: the emulated reference build uses no OpenGL. */
