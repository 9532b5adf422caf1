/* Build shim: included but unused by the reference (misc/simpleNumerics.h). */
