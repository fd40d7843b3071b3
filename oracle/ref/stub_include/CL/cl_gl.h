/* empty stand-in: no OpenCL-GL interop in the reference build */
