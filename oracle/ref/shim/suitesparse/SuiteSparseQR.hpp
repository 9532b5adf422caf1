/* Build shim: the header the reference includes here is not needed by its dense path. */
