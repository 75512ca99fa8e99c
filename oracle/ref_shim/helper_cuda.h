/* Empty stand-in for the CUDA samples header included by the reference. */
