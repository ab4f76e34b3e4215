// Empty stand-in: the reference includes it (tensor.h:5) but uses nothing from it.
