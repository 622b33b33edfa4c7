/* Empty stand-in: the reference includes <cblas.h> (test.cu:1, include/analysis.h:3) but calls no cblas routine. */
#pragma once
