

Bin/rtm.x:   lin7@cees-gpu   Fri Aug 14 13:18:48 2015
		n1=45
		o1=0
		d1=1
		sets next: in="/data/lin7/filter.H@"
		data_format="xdr_float"
