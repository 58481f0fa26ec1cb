/* Test-infrastructure stand-in: io/io.h includes <bodies.h>, which the grid and
 * body parsers do not use. */
#pragma once
