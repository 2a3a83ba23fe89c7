/* Places the zero guard (ref_guard.c) immediately in front of the reference's
 * CRC table in oracle/_ref/libsymref.so; see ref_guard.c. */
SECTIONS {
  .rodata.symref : { KEEP(*(.rodata.symref_guard)) *(.rodata._ZN12_GLOBAL__N_1L9crc64_tabE) }
} INSERT BEFORE .rodata;
