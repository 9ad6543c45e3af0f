/* Empty stand-in for linal's array.h (included by src/impl/deriv_impl.h). */
