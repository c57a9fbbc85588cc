/* Empty stand-in for the CUDPP header: the reference's loader and CPU
 * validator (read_input.cu, validate.cu) include it through common.h but use
 * no CUDPP symbol. */
#pragma once
