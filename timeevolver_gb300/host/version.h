// version.h -- API version of the TimeEvolver interface this library provides
// (the reference's core/version.h numbering: 201 = 2.0.1).
#pragma once
#define TIMEEVOLVER_VERSION 201
#define TIMEEVOLVER_VERSION_STRING "2_0_1"
