// pg_types.h -- integer types shared by host and device code.
#pragma once
typedef unsigned long long u64;
typedef unsigned int u32;
typedef unsigned short u16;
