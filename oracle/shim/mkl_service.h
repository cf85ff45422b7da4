/* Empty stand-in for MKL's service header (included by the reference's core.cpp:2). */
#pragma once
