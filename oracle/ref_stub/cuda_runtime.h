/* empty stand-in: oracle/ref_shim.h supplies the CUDA runtime pieces the reference API files use */
