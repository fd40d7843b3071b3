/* empty stand-in: no GLX in the reference build */
