/* empty: the reference includes this header but uses none of it */
